"""Lennard-Jones with a cutoff through the device cell list (an extension:
the reference's LjNd sums every pair).

* The pair set is bit-exact: the pairs the device's cell list evaluates at
  FP32-rounded coordinates equal a brute-force CPU enumeration testing
  r^2 < rc^2 on the same FP64 r^2 ((dx^2 + dy^2) + dz^2, one rounding per
  operation) of the same FP32 values, at N = 13 ... 5000, in 2-D and 3-D,
  with pairs placed exactly at rc (left out: the test is strict) and just
  inside it.
* Energies and gradients match the oracle restated with the same cutoff:
  the FP64 evaluation to 1e-12, the FP32 stage's kernels (whole GPU and one
  CTA) to the FP32-stage tolerances.
* Minimisations with a cutoff end at minima under the oracle.
"""
import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests.workloads import Rng, lj_cluster

pytestmark = pytest.mark.gpu

RC = 2.5


def brute_pairs(x, nd, rc):
    """Pairs i < j with r^2 < rc^2, r^2 in FP64 of the FP32-rounded values."""
    p = np.asarray(x, np.float32).astype(np.float64).reshape(-1, nd)
    n = p.shape[0]
    rc2 = rc * rc
    out = []
    for i0 in range(0, n, 512):
        a = p[i0:i0 + 512]
        d = [a[:, None, k] - p[None, :, k] for k in range(nd)]
        r2 = d[0] * d[0] + d[1] * d[1]
        if nd == 3:
            r2 = r2 + d[2] * d[2]
        ii, jj = np.nonzero(r2 < rc2)
        ii = ii + i0
        keep = jj > ii
        out.append(np.stack([ii[keep], jj[keep]], axis=1))
    q = np.concatenate(out) if out else np.zeros((0, 2), int)
    order = np.lexsort((q[:, 1], q[:, 0]))
    return q[order].astype(np.int32)


def with_edge_pairs(x, nd, rc):
    """x with pairs of particles appended at exactly rc and just inside it
    (FP32-exact offsets: 2.5 = |(1.5, 2.0)| too), far from the cluster and
    from each other."""
    pts = list(np.asarray(x).reshape(-1, nd))
    base = np.floor(pts[0]) + 40.0
    offs = [(rc, 0.0, 0.0), (1.5, 2.0, 0.0), (0.0, 1.5, 2.0), (rc * (1 - 2 ** -10), 0.0, 0.0)]
    pts.append(base[:nd].copy())
    for k, o in enumerate(offs):
        q = base[:nd] + np.array(o[:nd]) + np.array([0.0] * (nd - 1) + [10.0 * (k + 1)])
        pts.append(q)
        pts.append(q - np.array(o[:nd]))
    return np.asarray(pts).ravel()


@pytest.mark.parametrize("n,nd", [(13, 3), (256, 3), (1000, 3), (5000, 3), (400, 2)])
def test_pair_set_bit_exact(n, nd):
    x = with_edge_pairs(lj_cluster(n, seed=n, ndim=nd), nd, RC)
    inst = runtime.Instance(abi.lj(ndim=nd, cutoff=RC), x)
    dev = inst.cutoff_pairs(x)
    ref = brute_pairs(x, nd, RC)
    assert dev.shape == ref.shape, (dev.shape, ref.shape)
    assert np.array_equal(dev, ref)
    # pairs exactly at rc are out, the one just inside is in
    m = x.size // nd
    got = {tuple(p) for p in dev.tolist()}
    assert (m - 2, m - 1) in got
    assert (m - 8, m - 7) not in got
    assert (m - 6, m - 5) not in got
    if nd == 3:
        assert (m - 4, m - 3) not in got


def test_pair_set_far_flung_and_clamped():
    # particles far apart (cell indices beyond the clamp) next to a cluster
    rng = Rng(17)
    x = np.concatenate([lj_cluster(300, seed=5), rng.uniform(30) * 4e7 - 2e7,
                        [1e8, 1e8, 1e8, 1e8, 1e8, 1e8 + 2.0]])
    inst = runtime.Instance(abi.lj(cutoff=RC), x)
    assert np.array_equal(inst.cutoff_pairs(x), brute_pairs(x, 3, RC))


@pytest.mark.parametrize("n,seed", [(256, 0), (1000, 3), (3000, 4)])
def test_energy_gradient_matches_oracle(n, seed):
    p = abi.lj(cutoff=RC)
    x = lj_cluster(n, seed=seed)
    inst = runtime.Instance(p, x)
    ora = Oracle(p, x)
    e, g = inst.energy_gradient()
    eo, go = ora.energy_gradient()
    assert abs(e - eo) <= 1e-12 * abs(eo)
    assert np.max(np.abs(g - go)) <= 1e-12 * np.max(np.abs(go))
    x32 = np.asarray(x, np.float32).astype(np.float64)
    eo32, go32 = ora.energy_gradient(x32)
    for path in (abi.EVAL_FP32_GRID, abi.EVAL_FP32_CTA):
        e32, g32 = inst.eval_kernel(path, x)
        assert abs(e32 - eo32) <= 2e-6 * abs(eo32), path
        assert np.max(np.abs(g32 - go32)) <= 1e-5 * np.max(np.abs(go32)), path
    for path in (abi.EVAL_FP64S_GRID, abi.EVAL_FP64S_CTA):
        e64, g64 = inst.eval_kernel(path, x)
        assert abs(e64 - eo) <= 1e-12 * abs(eo), path
        assert np.max(np.abs(g64 - go)) <= 2e-7 * np.max(np.abs(go)), path


def test_cutoff_beyond_cluster_equals_all_pairs():
    x = lj_cluster(64, seed=9)
    e_all, g_all = runtime.Instance(abi.lj(), x).energy_gradient()
    e_cut, g_cut = runtime.Instance(abi.lj(cutoff=1e3), x).energy_gradient()
    assert abs(e_cut - e_all) <= 1e-12 * abs(e_all)
    assert np.max(np.abs(g_cut - g_all)) <= 1e-12 * np.max(np.abs(g_all))


def test_nan_coordinate_gives_nan_energy():
    x = lj_cluster(50, seed=2)
    x[10] = np.nan
    e, g = runtime.Instance(abi.lj(cutoff=RC), x).energy_gradient()
    assert np.isnan(e)
    assert np.isnan(g[9:12]).all()


@pytest.mark.parametrize("how", ["grid", "batch"])
def test_minimise_with_cutoff(how):
    p = abi.lj(cutoff=RC)
    x0 = lj_cluster(600, seed=21)
    inst = runtime.Instance(p, x0)
    mp = abi.minimiser("lbfgs", m=5, tol=1e-5, max_iter=20000)
    if how == "grid":
        r = inst.minimise(mp)
    else:
        b = runtime.Batch()
        b.add(inst, mp)
        r = b.run()[0]
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    ora = Oracle(p, x0)
    e, g = ora.energy_gradient(inst.coords)
    assert np.sqrt(np.mean(g ** 2)) < 1e-5
    assert abs(r.energy - e) <= 1e-8 * abs(e)


def test_invalid_cutoff_rejected():
    x = lj_cluster(13, seed=1)
    for rc in (-1.0, float("inf"), float("nan")):
        with pytest.raises(runtime.MinimGpuError) as e:
            runtime.Instance(abi.lj(cutoff=rc), x)
        assert e.value.code == abi.ERR_INVALID
    with pytest.raises(runtime.MinimGpuError):
        runtime.Instance(abi.lj(), x).cutoff_pairs(x)
