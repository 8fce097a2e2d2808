"""Per-evaluation parity on the GPU: energy and constrained gradient through
the C ABI (FP64 evaluation) against the FP64 C oracle, for every potential
and the optional PhaseField / BarAndHinge terms, plus State::applyConstraints."""
import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests.workloads import Rng, lj_cluster, pf_noise, pf_simplex, sheet

pytestmark = pytest.mark.gpu

REL = 1e-12  # FP64 evaluation: rounding-level agreement


def _cmp(p, x0, x=None, fixed=None, rel=REL):
    inst = runtime.Instance(p, x0, fixed=fixed)
    ora = Oracle(p, x0, fixed=fixed)
    e, g = inst.energy_gradient(x)
    eo, go = ora.energy_gradient(x)
    scale_e = max(abs(eo), 1e-300)
    assert abs(e - eo) <= rel * scale_e + 1e-14, (e, eo)
    gs = max(np.max(np.abs(go)), 1e-300)
    assert np.max(np.abs(g - go)) <= rel * gs + 1e-14, np.max(np.abs(g - go)) / gs
    return inst, ora


def test_lj_pair_kat():
    # reference test/unit/State_test.cpp:33-51
    inst = runtime.Instance(abi.lj(), [0, 0, 0, 2, 0, 0])
    e, g = inst.energy_gradient()
    assert e == pytest.approx(-63.0 / 1024, rel=1e-15)
    assert np.allclose(g, [-93.0 / 512, 0, 0, 93.0 / 512, 0, 0], atol=1e-15)


@pytest.mark.parametrize("n,ndim", [(13, 3), (64, 3), (400, 3), (1500, 3), (30, 2)])
def test_lj_random(n, ndim):
    x = lj_cluster(n, seed=n, ndim=ndim)
    _cmp(abi.lj(ndim=ndim, sigma=1.1, epsilon=0.7), x)


def test_lj_fixed_dofs():
    x = lj_cluster(20, seed=1)
    _cmp(abi.lj(), x, fixed=[0, 1, 2, 17, 40])


@pytest.mark.parametrize("grid", [(6, 5, 4), (1, 1, 7), (2, 3, 1), (16, 16, 16)])
def test_pf_binary(grid):
    x = pf_noise(grid, seed=2, amp=0.5)
    _cmp(abi.phase_field(grid, interface_size=1.3, surface_tension=0.7), x)


def test_pf_binary_pressure_resolution():
    x = pf_noise((5, 6, 7), seed=3, amp=0.9)
    _cmp(abi.phase_field((5, 6, 7), resolution=2.0, pressure=[1.5]), x)


def _walls(shape):
    s = np.zeros(shape, np.uint8)
    s[:, 0, :] = 1
    return s


def test_pf_binary_solid_contact_force():
    shape = (9, 8, 5)
    solid = np.zeros(shape, np.uint8)
    solid[3:5, 2:4, 1:3] = 1
    solid[:, 0, :] = 1
    ca = Rng(4).uniform(int(np.prod(shape))) * 120 + 30
    x = pf_noise(shape, seed=4, amp=0.9)
    _cmp(abi.phase_field(shape, solid=solid.ravel(), contact_angle=ca, force=[0.1, -0.3, 0.2],
                         pressure=[0.4]), x)


@pytest.mark.parametrize("density", ["hard", "soft", "none", "fixed"])
def test_pf_ternary(density):
    shape = (12, 10, 1)
    x = pf_simplex(shape, 3, seed=5)
    p = abi.phase_field(shape, nfluid=3, solid=_walls(shape).ravel(), volume_fixed=True,
                        density_constraint=density, surface_tension=[1.0, 0.8, 1.2],
                        pressure=[0, 0.3, 0], force=[[0, -1, 0], [0.2, 0, 0], [0, 0, 0]],
                        confinement=[0, 1.0, 0])
    inst, ora = _cmp(p, x)
    v = Rng(6).normal(x.size)
    assert np.allclose(inst.apply_constraints(v), ora.apply_constraints(v), rtol=1e-12, atol=1e-12)


def test_pf_fixfluid_and_node_tension():
    shape = (6, 5, 3)
    ng = int(np.prod(shape))
    st = 0.5 + Rng(7).uniform(ng * 2)
    x = pf_simplex(shape, 2, seed=7)
    _cmp(abi.phase_field(shape, nfluid=2, surface_tension=st, fix_fluid=[1, 0],
                         density_constraint="none"), x)


def test_bah_two_triangles():
    x0 = np.array([-1, 0, 1, 0, -np.sqrt(2), 0, 0, np.sqrt(2), 0, 1, 0, 1.0])
    p = abi.bar_and_hinge(triangulation=[[0, 1, 2], [1, 3, 2]], rigidity=(100, 1))
    x = x0 + Rng(8).normal(12) * 0.2
    _cmp(p, x0, x)


@pytest.mark.parametrize("k", [6, 20])
def test_bah_sheet(k):
    flat, tris, pert = sheet(k, seed=k)
    _cmp(abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01)), flat, pert)


def test_bah_thickness_force_wall_fixed():
    flat, tris, pert = sheet(8, seed=9)
    p = abi.bar_and_hinge(triangulation=tris, thickness=0.1, modulus=2.0, force=[0, 0, -0.01],
                          wall=True, wall_adhesion=True, wall_params=(1e-3, 0.5))
    _cmp(p, flat, pert - 0.05, fixed=list(range(9)))
