"""One instance on a thread-block cluster of several CTAs (the batch path's
multi-SM shape, `minim_gpu_batch_run_shape` and the autotuner's cluster
candidates), through the C ABI:

* every cluster size ends at a minimum under the oracle, for the general
  PhaseField, BarAndHinge and Lennard-Jones kernels;
* a one-CTA shape through the shape entry point is bitwise the plain batch;
* an instance's result with a cluster shape is the same alone and in a
  batch with other instances and shapes;
* the autotuner times the cluster candidates of large keys.
"""
import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests.workloads import lj_cluster, pf_simplex, sheet

pytestmark = pytest.mark.gpu


def _run(insts, mp, threads=0, ctas=0):
    b = runtime.Batch()
    for i in insts:
        b.add(i, mp)
    return b.run(threads=threads, ctas=ctas)


def _check_min(p, x0, x, r, tol, start=None):
    ora = Oracle(p, x0)
    e, g = ora.energy_gradient(x)
    assert np.sqrt(np.mean(g ** 2)) < tol
    e0 = ora.energy(start if start is not None else x0)
    assert abs(r.energy - e) <= 1e-8 * max(abs(e), abs(e0))


@pytest.mark.parametrize("ctas", [1, 2, 4, 8])
def test_pf_cluster_sizes(ctas):
    grid = (128, 128, 1)
    p = abi.phase_field(grid, nfluid=3, volume_fixed=True)
    x0 = pf_simplex(grid, 3, seed=41)
    inst = runtime.Instance(p, x0)
    r = _run([inst], abi.minimiser("lbfgs", tol=1e-7, max_iter=20000), threads=512, ctas=ctas)[0]
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    _check_min(p, x0, inst.coords, r, 1e-7)


@pytest.mark.parametrize("ctas", [2, 8])
def test_bah_cluster(ctas):
    flat, tris, pert = sheet(60, seed=42)
    p = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01))
    inst = runtime.Instance(p, flat)
    inst.coords = pert
    r = _run([inst], abi.minimiser("lbfgs", tol=1e-7, max_iter=50000), threads=512, ctas=ctas)[0]
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    _check_min(p, flat, inst.coords, r, 1e-7, start=pert)


@pytest.mark.parametrize("ctas", [1, 4])
def test_lj_cluster(ctas):
    p = abi.lj()
    x0 = lj_cluster(700, seed=43)
    inst = runtime.Instance(p, x0)
    r = _run([inst], abi.minimiser("lbfgs", m=5, tol=1e-6, max_iter=50000), threads=256, ctas=ctas)[0]
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    _check_min(p, x0, inst.coords, r, 1e-6)


def test_one_cta_shape_is_the_plain_batch():
    grid = (64, 64, 1)
    p = abi.phase_field(grid, nfluid=3, volume_fixed=True)
    x0 = pf_simplex(grid, 3, seed=44)
    mp = abi.minimiser("lbfgs", tol=1e-7, max_iter=20000)
    a, b = runtime.Instance(p, x0), runtime.Instance(p, x0)
    ra = _run([a], mp, threads=512)[0]
    rb = _run([b], mp, threads=512, ctas=1)[0]
    assert (ra.iter, ra.evals, ra.energy) == (rb.iter, rb.evals, rb.energy)
    assert np.array_equal(a.coords, b.coords)


def test_cluster_result_same_alone_and_in_mix():
    grid = (128, 96, 1)
    p = abi.phase_field(grid, nfluid=3, volume_fixed=True)
    x0 = pf_simplex(grid, 3, seed=45)
    mp = abi.minimiser("lbfgs", tol=1e-7, max_iter=20000)
    a = runtime.Instance(p, x0)
    ra = _run([a], mp, threads=512, ctas=4)[0]
    b = runtime.Instance(p, x0)
    others = [runtime.Instance(abi.phase_field((g, g, 1), nfluid=3, volume_fixed=True),
                               pf_simplex((g, g, 1), 3, seed=46 + g)) for g in (40, 96, 64)]
    res = _run([others[0], b] + others[1:], mp, threads=512, ctas=4)
    rb = res[1]
    assert ra.status == abi.RES_CONVERGED
    assert (ra.iter, ra.evals, ra.energy) == (rb.iter, rb.evals, rb.energy)
    assert np.array_equal(a.coords, b.coords)


def test_shape_entry_rejects_bad_shapes():
    inst = runtime.Instance(abi.lj(), lj_cluster(20, seed=1))
    b = runtime.Batch()
    b.add(inst, abi.minimiser("lbfgs", tol=1e-6))
    for threads, ctas in [(512, 1), (100, 1), (256, 9), (256, 0)]:
        if ctas == 0:
            continue
        with pytest.raises(runtime.MinimGpuError) as e:
            b.run(threads=threads, ctas=ctas)
        assert e.value.code == abi.ERR_INVALID


def test_tuner_times_cluster_candidates():
    grid = (256, 256, 1)
    p = abi.phase_field(grid, nfluid=3, volume_fixed=True)
    insts = [runtime.Instance(p, pf_simplex(grid, 3, seed=50 + i)) for i in range(3)]
    mp = abi.minimiser("lbfgs", tol=1e-7, max_iter=20000)
    res = _run(insts, mp)
    for r in res:
        assert r.status == abi.RES_CONVERGED, r.as_dict()
    rows = [t for t in runtime.tune_table() if t["kind"] == "pf" and t["bucket"] >= 2 and t["measured"]]
    assert rows
    for t in rows:
        # 256 / 512 threads on one CTA (the sample), clusters of 2 / 4 / 8
        # (the largest instance alone), and the one-CTA time of that instance
        ms = t["candidate_ms"]
        assert len(ms) == 6 and all(v > 0 for v in ms)
        assert t["ctas"] in (1, 2, 4, 8)
        if t["ctas"] > 1:
            c = {2: 2, 4: 3, 8: 4}[t["ctas"]]
            assert ms[5] >= 0.5 * t["ctas"] * ms[c]
