"""Error bounds of the engine's hand-written arithmetic helpers against
CUDA's own correctly rounded operations, over a sweep of inputs
(tests/cuda/math_probe.cu, compiled here with nvcc for sm_103a):

* rcp_nr -- the hardware reciprocal approximation refined by one
  Newton-Raphson step (the FP32 Lennard-Jones pair term): within 1 ulp of
  __frcp_rn;
* df_split_bits -- a double split into two FP32 values by its bits: relative
  error below 2^-46;
* df_rcp -- the FP32 reciprocal refined by one Newton step in double-float:
  relative error below 2^-44 against 1.0 / x in FP64;
* the double-float square root (one Newton step from sqrtf, the BarAndHinge
  FP64 stage): relative error below 2^-44 against sqrt in FP64;
* the double-float product (Dekker / FMA): relative error below 2^-44;
* the Lennard-Jones pair terms' double-float (DFl): the reciprocal with its
  residual from fused multiply-adds, relative error below 2^-44; the sum,
  error below 2^-45 of the operands' magnitudes.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("probe") / "libmath_probe.so")
    nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++20", "-shared",
                    "-Xcompiler", "-fPIC", "-I" + os.path.join(REPO, "include"),
                    "-I" + os.path.join(REPO, "minim_gb300", "csrc"),
                    os.path.join(REPO, "tests", "cuda", "math_probe.cu"), "-o", out], check=True)
    lib = C.CDLL(out)
    dp = C.POINTER(C.c_double)
    lib.math_probe.argtypes = [dp, dp, dp, C.c_int]

    def run(x, y):
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        o = np.zeros((x.size, 12))
        assert lib.math_probe(x.ctypes.data_as(dp), y.ctypes.data_as(dp), o.ctypes.data_as(dp), x.size) == 0
        return o
    return run


def _inputs():
    rng = np.random.default_rng(5)
    # magnitudes 2^-60 .. 2^60 with random mantissas, both signs, plus the
    # Lennard-Jones r^2 range and exact powers of two
    e = rng.uniform(-60, 60, 200000)
    m = rng.uniform(1, 2, e.size)
    x = np.ldexp(m, np.floor(e).astype(int)) * np.where(rng.uniform(size=e.size) < 0.5, -1, 1)
    r2 = rng.uniform(1e-5, 1e4, 100000)
    p2 = np.ldexp(1.0, np.arange(-60, 61))
    return np.concatenate([x, r2, p2, -p2])


def test_rcp_nr_within_one_ulp(probe):
    x = _inputs()
    o = probe(x, x)
    nr, rn = o[:, 0].astype(np.float32), o[:, 1].astype(np.float32)
    ulps = np.abs(nr.view(np.int32).astype(np.int64) - rn.view(np.int32).astype(np.int64))
    assert ulps.max() <= 1, ulps.max()
    assert np.mean(ulps == 0) > 0.5


def test_double_float_helpers(probe):
    x = _inputs()
    y = np.random.default_rng(6).permutation(x)
    o = probe(x, y)
    rel = lambda a, b: np.abs(a - b) / np.abs(b)
    assert rel(o[:, 2], x).max() < 2.0 ** -46
    assert rel(o[:, 3], o[:, 4]).max() < 2.0 ** -44
    pos = x > 0
    assert rel(o[pos, 5], o[pos, 6]).max() < 2.0 ** -44
    prod = x * y
    ok = (np.abs(prod) > 2.0 ** -80) & (np.abs(prod) < 2.0 ** 80)
    assert rel(o[ok, 7], prod[ok]).max() < 2.0 ** -44


def test_lj_double_float(probe):
    x = _inputs()
    y = np.random.default_rng(7).permutation(x)
    o = probe(x, y)
    assert (np.abs(o[:, 8] - o[:, 4]) / np.abs(o[:, 4])).max() < 2.0 ** -44
    assert (np.abs(o[:, 9] - o[:, 10]) / o[:, 11]).max() < 2.0 ** -45
