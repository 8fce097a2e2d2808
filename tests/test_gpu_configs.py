"""The benchmark configurations themselves, minimised on the GPU and checked
under the FP64 oracle (with the oracle's own run of the reference algorithm
recorded beside the GPU's where it is cheap):

* the plain Lennard-Jones cluster: N = 256 from seed 0, Lbfgs(m = 5) to RMS
  < 1e-6, on the whole GPU and in a batch;
* the 192^3 binary PhaseField of the single-instance workload, Lbfgs(m = 10)
  to RMS < 1e-7 (the stepped graph's FP32 stage, then FP64);
* a sample of the batched Lennard-Jones workload (N ~ U{13..400}, per-instance
  seeds): its Lbfgs half in one batch.

LJ landscapes are chaotic, so a GPU run and the oracle's may reach different
minima; the check is that the GPU's point is a minimum under the oracle and
that the GPU's energy is the oracle's energy there.  With MINIM_PARITY_LOG
set, both runs' iteration counts and energies are appended to that file.
"""
import json
import os

import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests.workloads import Rng, lj_cluster, pf_noise

pytestmark = pytest.mark.gpu


def _log(**kw):
    fn = os.environ.get("MINIM_PARITY_LOG")
    if fn:
        with open(fn, "a") as f:
            f.write(json.dumps(kw) + "\n")


def _check(p, x0, x, r, tol, floor=False):
    ora = Oracle(p, x0)
    e, g = ora.energy_gradient(x)
    rms = float(np.sqrt(np.mean(g ** 2)))
    assert rms < tol, rms
    scale = max(abs(e), abs(ora.energy(x0))) if floor else abs(e)
    assert abs(r.energy - e) <= 1e-8 * scale, (r.energy, e)
    return e, rms


@pytest.mark.parametrize("how", ["grid", "batch"])
def test_plain_lj_cluster_256(how):
    p = abi.lj()
    x0 = lj_cluster(256, seed=0)
    mp = abi.minimiser("lbfgs", m=5, tol=1e-6)
    inst = runtime.Instance(p, x0)
    if how == "grid":
        r = inst.minimise(mp)
    else:
        b = runtime.Batch()
        b.add(inst, mp)
        r = b.run()[0]
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    e, rms = _check(p, x0, inst.coords, r, 1e-6)
    ro = Oracle(p, x0).minimise(mp)
    assert ro.status == abi.RES_CONVERGED
    _log(case="lj256_seed0", path=how, gpu_iter=r.iter, gpu_energy=r.energy, oracle_iter=ro.iter,
         oracle_energy=ro.energy, oracle_rms_at_gpu_point=rms)


def test_pf_binary_192_workload():
    grid = (192, 192, 192)
    p = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0)
    x0 = pf_noise(grid, seed=0, amp=0.05)
    inst = runtime.Instance(p, x0)
    r = inst.minimise(abi.minimiser("lbfgs", m=10, tol=1e-7))
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    e, rms = _check(p, x0, inst.coords, r, 1e-7, floor=True)
    _log(case="pf192", gpu_iter=r.iter, gpu_fp64_iters=r.fp64_iters, gpu_energy=r.energy, oracle_energy_at_x=e,
         oracle_rms_at_x=rms)


def test_batched_lj_sample():
    rng = Rng(12345)
    sizes = 13 + (rng.uniform(4096) * (400 - 13 + 1)).astype(int)
    idx = list(range(2048, 2048 + 12))  # the Lbfgs half, per-instance seeds = index
    p = abi.lj()
    mp = abi.minimiser("lbfgs", m=5, tol=1e-6)
    insts = [runtime.Instance(p, lj_cluster(int(sizes[i]), seed=i)) for i in idx]
    b = runtime.Batch()
    for inst in insts:
        b.add(inst, mp)
    res = b.run()
    for i, inst, r in zip(idx, insts, res):
        assert r.status == abi.RES_CONVERGED, (i, r.as_dict())
        _check(p, lj_cluster(int(sizes[i]), seed=i), inst.coords, r, 1e-6)
