"""PhaseFieldUnstructured on the GPU: the element form of the phase field
(src/potentials/PhaseFieldUnstructured.cpp) evaluated by the PhaseField
sweep with its element semantics, against the FP64 oracle and against
fixtures produced by the reference library itself (tests/golden/pfu_*.npz).

  * evaluation (FP64): energy and constrained gradient to rounding, and
    State::applyConstraints, for every element type, both fixed-volume forms
    (penalty), all four density constraints and user-fixed degrees of freedom;
  * minimisation (mixed precision): the reference's minimum, energy to 1e-8
    relative, a minimum under the FP64 gradient;
  * a binary field with none of the optional terms has the same energy as
    PhaseField and runs the same fast path.
"""
import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests import golden_io as G
from tests.workloads import pf_noise, pf_simplex

pytestmark = pytest.mark.gpu

EG = G.load("pfu_eg.npz")
MIN = G.load("pfu_min.npz")


@pytest.mark.parametrize("c", EG, ids=G.case_ids(EG))
def test_eval_matches_reference(c):
    p = G.params_from("pfu", c["params_kw"])
    fixed = c["fixed"] if c["fixed"].size else None
    inst = runtime.Instance(p, c["x0"], fixed=fixed)
    e, g = inst.energy_gradient(c["x"])
    e_ref = float(c["energy"])
    assert abs(e - e_ref) <= 1e-12 * max(abs(e_ref), 1.0), (e, e_ref)
    gs = max(np.max(np.abs(c["gradient"])), 1e-300)
    assert np.max(np.abs(g - c["gradient"])) <= 1e-12 * gs
    eo, go = Oracle(p, c["x0"], fixed=fixed).energy_gradient(c["x"])
    assert abs(e - eo) <= 1e-12 * max(abs(eo), 1.0)
    assert np.max(np.abs(g - go)) <= 1e-12 * gs
    v = inst.apply_constraints(c["v"])
    assert np.allclose(v, c["v_constrained"], rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("c", MIN, ids=G.case_ids(MIN))
def test_minimise_reaches_reference_minimum(c):
    p = G.params_from("pfu", c["params_kw"])
    inst = runtime.Instance(p, c["x0"])
    inst.coords = c["start"]
    mkw = c["minimiser_kw"]
    r = inst.minimise(G.mp_from(mkw))
    assert r.status == int(c["status"]) == abi.RES_CONVERGED, r.as_dict()
    ora = Oracle(p, c["x0"])
    e, g = ora.energy_gradient(inst.coords)
    assert np.sqrt(np.mean(g ** 2)) < mkw["tol"]
    e_init = ora.energy(c["start"])
    e_ref = float(c["energy"])
    assert abs(r.energy - e) <= 1e-8 * max(abs(e), abs(e_init))
    assert abs(r.energy - e_ref) <= 1e-8 * max(abs(e_ref), abs(e_init)), (r.energy, e_ref)


@pytest.mark.parametrize("grid", [(16, 12, 8), (10, 9, 7)])
def test_binary_equals_phase_field(grid):
    x0 = pf_noise(grid, seed=41, amp=0.6)
    a = runtime.Instance(abi.phase_field_unstructured(grid), x0)
    b = runtime.Instance(abi.phase_field(grid), x0)
    ea, ga = a.energy_gradient()
    eb, gb = b.energy_gradient()
    assert ea == eb and np.array_equal(ga, gb)
    mp = abi.minimiser("lbfgs", m=10, tol=1e-7)
    ra, rb = a.minimise(mp), b.minimise(mp)
    assert ra.status == rb.status == abi.RES_CONVERGED
    assert ra.iter == rb.iter and ra.energy == rb.energy
    assert np.array_equal(a.coords, b.coords)


def test_ternary_penalty_batch():
    """Batched minimisation of ternary fields with the volume penalty and
    the hard density constraint: a minimum under the FP64 gradient, and the
    per-node density stays 1."""
    shape = (20, 20, 1)
    b = runtime.Batch()
    insts = []
    for s in range(4):
        p = abi.phase_field_unstructured(shape, nfluid=3, volume_fixed=True, vol_const=0.01)
        x0 = pf_simplex(shape, 3, seed=60 + s)
        inst = runtime.Instance(p, x0)
        b.add(inst, abi.minimiser("lbfgs", tol=1e-6, max_iter=20000))
        insts.append((p, x0, inst))
    for (p, x0, inst), r in zip(insts, b.run()):
        assert r.status in (abi.RES_CONVERGED, abi.RES_MAXITER), r.as_dict()
        x = inst.coords
        ora = Oracle(p, x0)
        e = ora.energy(x)
        assert abs(r.energy - e) <= 1e-8 * max(abs(e), abs(ora.energy(x0)))
        assert np.allclose(x.reshape(-1, 3).sum(axis=1), 1.0, atol=1e-6)
        if r.status == abi.RES_CONVERGED:
            assert np.sqrt(np.mean(ora.gradient(x) ** 2)) < 1e-6


def test_invalid_arguments():
    with pytest.raises(runtime.MinimGpuError):
        runtime.Instance(abi.phase_field_unstructured((4, 4, 1), nfluid=2, density_constraint="soft"),
                         np.full(32, 0.5))
    with pytest.raises(runtime.MinimGpuError):
        runtime.Instance(abi.phase_field_unstructured((4, 4, 1), surface_tension=np.ones(16)), np.zeros(16))
