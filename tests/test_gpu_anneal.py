"""Anneal on the GPU (src/minimisers/Anneal.cpp): the device run against the
FP64 oracle drawing the same counter-based random numbers (the oracle's
Anneal is pinned to the reference library by tests/test_oracle_golden.py,
where it draws from rand() in the reference's order).

Every iteration's Metropolis decision depends on the energy at the moved
point; the device sums energies in another order than the oracle, so the two
agree to rounding and take the same decisions (a flip needs a random number
within rounding of the acceptance threshold).  The runs must therefore end
at the same iteration with the same coordinates.
"""
import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests import golden_io as G
from tests.workloads import lj_cluster, pf_noise

pytestmark = pytest.mark.gpu

CASES = G.load("anneal_min.npz")


def _same_run(r, ro, x, xo):
    assert r.status == ro.status and r.iter == ro.iter, (r.as_dict(), ro.as_dict())
    assert abs(r.energy - ro.energy) <= 1e-12 * max(abs(ro.energy), 1.0)
    assert np.max(np.abs(x - xo)) <= 1e-12 * max(np.max(np.abs(xo)), 1.0)


@pytest.mark.parametrize("c", CASES, ids=G.case_ids(CASES))
def test_single_instance_follows_oracle(c):
    p = G.params_from(c["kind"], c["params_kw"])
    mp = G.mp_from(c["minimiser_kw"])
    inst = runtime.Instance(p, c["x0"])
    inst.coords = c["start"]
    r = inst.minimise(mp)
    ora = Oracle(p, c["x0"])
    ora.coords = c["start"]
    ro = ora.minimise(mp)
    _same_run(r, ro, inst.coords, ora.coords)
    assert r.evals == ro.evals


def test_batch_follows_oracle():
    """Several annealing runs (different sizes, seeds, schedules) in one
    batch: each follows its own oracle run."""
    b = runtime.Batch()
    items = []
    for k, n in enumerate([13, 38, 55, 13]):
        p = abi.lj()
        x0 = lj_cluster(n, seed=100 + k)
        kw = dict(temp_init=0.3, displacement=0.02, max_iter=1500, seed=500 + k)
        if k == 3:
            kw.update(temp_schedule=np.geomspace(0.3, 1e-3, 1000), max_rejections=200)
        mp = abi.minimiser("anneal", **kw)
        inst = runtime.Instance(p, x0)
        b.add(inst, mp)
        items.append((p, x0, mp, inst))
    for (p, x0, mp, inst), r in zip(items, b.run()):
        ora = Oracle(p, x0)
        ro = ora.minimise(mp)
        _same_run(r, ro, inst.coords, ora.coords)


def test_grid_instance_follows_oracle():
    """A 48^3 binary phase field (the multi-block grid path)."""
    shape = (48, 48, 48)
    p = abi.phase_field(shape)
    x0 = pf_noise(shape, seed=7, amp=0.5)
    mp = abi.minimiser("anneal", temp_init=1e-3, displacement=1e-3, max_iter=40, seed=77)
    inst = runtime.Instance(p, x0)
    r = inst.minimise(mp)
    ora = Oracle(p, x0)
    ro = ora.minimise(mp)
    _same_run(r, ro, inst.coords, ora.coords)


def test_seed_determinism():
    p = abi.lj()
    x0 = lj_cluster(20, seed=3)
    out = []
    for seed in (5, 5, 6):
        inst = runtime.Instance(p, x0)
        r = inst.minimise(abi.minimiser("anneal", temp_init=0.5, displacement=0.05, max_iter=300, seed=seed))
        out.append((r.energy, inst.coords))
    assert out[0][0] == out[1][0] and np.array_equal(out[0][1], out[1][1])
    assert not np.array_equal(out[0][1], out[2][1])


def test_max_rejections_converges():
    p = abi.lj()
    x0 = lj_cluster(13, seed=5)
    inst = runtime.Instance(p, x0)
    r = inst.minimise(abi.minimiser("anneal", temp_init=1e-4, displacement=0.05, max_rejections=20, seed=8))
    assert r.status == abi.RES_CONVERGED and r.iter < 100000
    assert r.energy <= Oracle(p, x0).energy()
