"""Known-answer tests of the reference's own unit tests, restated against
the oracle (the reference's gtest submodules are not vendored, so its tests
cannot run as they are):
  test/unit/State_test.cpp:33-51, PhaseField_test.cpp:31-108,130-201,
  Potential_test.cpp:10-63 (fixed-dof projection), Fire_test.cpp:25-52,
  PhaseFieldUnstructured_test.cpp:27-208."""
import numpy as np
import pytest

from minim_gb300 import abi
from oracle.oracle import Oracle


def test_lj_pair():
    o = Oracle(abi.lj(), [0, 0, 0, 2, 0, 0])
    e, g = o.energy_gradient()
    assert e == -63.0 / 1024
    assert np.allclose(g, [-93.0 / 512, 0, 0, 93.0 / 512, 0, 0], atol=1e-15)


def test_pf_bulk_constant():
    o = Oracle(abi.phase_field([1, 1, 1]), [1.0])
    k, kp, _, _ = o.pf_internals()
    assert k[0] == 3 and kp[0] == 3
    e, g = o.energy_gradient()
    assert e == 0 and np.allclose(g, [0])
    e, g = o.energy_gradient([0.1])
    assert e == pytest.approx(3.0 / 16 * 1.21 * 0.81)
    assert np.allclose(g, [-3.0 / 4 * 0.099], atol=1e-6)


@pytest.mark.parametrize("grid", [[5, 1, 1], [1, 5, 1], [1, 1, 5]])
def test_pf_gradient_solid_bounded(grid):
    o = Oracle(abi.phase_field(grid, solid=[1, 0, 0, 0, 1]), [0, -1, 0, 1, 0])
    e, g = o.energy_gradient()
    assert e == pytest.approx(3.0 / 16 + 2 * (3.0 / 4))
    assert np.allclose(g, [0, -1.5, 0, 1.5, 0], atol=1e-6)


@pytest.mark.parametrize("grid", [[3, 1, 1], [1, 3, 1], [1, 1, 3]])
def test_pf_gradient_periodic(grid):
    o = Oracle(abi.phase_field(grid, solid=[0, 1, 0]), [-1, 0, 1])
    e, g = o.energy_gradient()
    assert e == pytest.approx(3.0 / 4 * 4)
    assert np.allclose(g, [-3, 0, 3], atol=1e-6)


def test_pf_force():
    for f, gexp in [([-2, 0, 0], [-.5, -.5, -.5, -.5, .5, .5, .5, .5]),
                    ([0, -2, 0], [-.5, -.5, .5, .5, -.5, -.5, .5, .5]),
                    ([0, 0, -2], [-.5, .5, -.5, .5, -.5, .5, -.5, .5])]:
        o = Oracle(abi.phase_field([2, 2, 2], force=f), [1] * 8)
        e, g = o.energy_gradient()
        assert e == pytest.approx(0, abs=1e-12)
        assert np.allclose(g, gexp, atol=1e-6)
    o = Oracle(abi.phase_field([2, 2, 2], surface_tension=0, force=[-4, 0, 0]), [-1] * 4 + [1] * 4)
    e, g = o.energy_gradient()
    assert e == pytest.approx(8)
    assert np.allclose(g, [0, 0, 0, 0, 1, 1, 1, 1], atol=1e-6)


def test_pf_surface():
    o = Oracle(abi.phase_field([2, 1, 1], surface_tension=0, contact_angle=[90, 60], solid=[1, 0]),
               [0.0, 0.5])
    e, g = o.energy_gradient()
    assert e == pytest.approx(0.5 / np.sqrt(2.0) * (-27.0 / 24))
    assert np.allclose(g, [0, 0.5 / np.sqrt(2.0) * (-0.75)], atol=1e-6)


def test_pf_pressure():
    o = Oracle(abi.phase_field([6, 1, 1], solid=[1, 0, 0, 0, 0, 1], pressure=[10]), [1] * 6)
    e, g = o.energy_gradient()
    assert e == pytest.approx(-30)
    assert np.allclose(g, [0, -2.5, -5, -5, -2.5, 0], atol=1e-6)


def test_pf_resolution():
    o = Oracle(abi.phase_field([5, 1, 1], resolution=2, solid=[1, 0, 0, 0, 1]), [0, -1, 0, 1, 0])
    k, kp, _, _ = o.pf_internals()
    assert k[0] == 1.5 and kp[0] == 6
    e, g = o.energy_gradient()
    assert e == pytest.approx(1.5 / 16 * 8 + 2 * (6.0 / 4) * 2)
    assert np.allclose(g, [0, -6, 0, 6, 0], atol=1e-6)
    o = Oracle(abi.phase_field([2, 2, 2], resolution=2, surface_tension=0, force=[-4, 0, 0]),
               [-1] * 4 + [1] * 4)
    e, g = o.energy_gradient()
    assert e == pytest.approx(128)
    assert np.allclose(g, [0, 0, 0, 0, 16, 16, 16, 16], atol=1e-6)
    o = Oracle(abi.phase_field([2, 1, 1], resolution=2, surface_tension=0, solid=[1, 0],
                               contact_angle=[90, 60]), [0, 0.5])
    e, g = o.energy_gradient()
    assert e == pytest.approx(0.5 / np.sqrt(2.0) * (-27.0 / 24) * 4)
    o = Oracle(abi.phase_field([6, 1, 1], resolution=2, solid=[1, 0, 0, 0, 0, 1], pressure=[10]), [1] * 6)
    e, g = o.energy_gradient()
    assert e == pytest.approx(-240)
    assert np.allclose(g, [0, -20, -40, -40, -20, 0], atol=1e-6)


def test_pf_fix_fluid():
    o = Oracle(abi.phase_field([2, 2, 1], nfluid=3, density_constraint="none", fix_fluid=[1, 0, 0]),
               [1.0] * 12)
    g = o.gradient()
    assert np.all(g[0::3] == 0)


def test_fixed_dof_constraint():
    o = Oracle(abi.lj(), [0, 0, 0, 2, 0, 0], fixed=[1, 3])
    g = o.gradient()
    assert g[1] == 0 and g[3] == 0
    v = o.apply_constraints(np.arange(6.0) + 1)
    assert np.array_equal(v, [1, 0, 3, 0, 5, 6])


def test_fire_first_step():
    from tests.workloads import lj_cluster
    x0 = lj_cluster(8, seed=13)
    o = Oracle(abi.lj(), x0)
    g = o.gradient()
    o.minimise(abi.minimiser("fire", linesearch="backtracking", max_iter=0))
    dt = 0.1 / np.linalg.norm(g) ** 0.5
    assert np.allclose(o.coords, x0 - 0.5 * dt * dt * g, atol=1e-14)


def test_bah_hinge_minima():
    s2 = np.sqrt(2)
    dz = s2 / 2
    x0 = np.array([-1, 0, 1, 0, -s2, 0, 0, s2, 0, 1, 0, 1.0])
    cases = [(1e-6, [0, 0, 0.5 + dz, 0, -s2, 0.5 - dz, 0, s2, 0.5 - dz, 0, 0, 0.5 + dz]),
             (np.pi / 2, [-1, 0, 1, 0, -s2, 0, 0, s2, 0, 1, 0, 1]),
             (np.pi, [-s2, 0, 0.5, 0, -s2, 0.5, 0, s2, 0.5, s2, 0, 0.5]),
             (3 * np.pi / 2, [-1, 0, 0, 0, -s2, 1, 0, s2, 1, 1, 0, 0]),
             (2 * np.pi - 1e-6, [0, 0, 0.5 - dz, 0, -s2, 0.5 + dz, 0, s2, 0.5 + dz, 0, 0, 0.5 - dz])]
    for t0, exp in cases:
        o = Oracle(abi.bar_and_hinge(triangulation=[[0, 1, 2], [1, 3, 2]], rigidity=(100, 1), theta0=[t0]), x0)
        o.minimise(abi.minimiser("lbfgs"))
        assert np.allclose(o.coords, exp, atol=1e-4)


# ---- PhaseFieldUnstructured: test/unit/PhaseFieldUnstructured_test.cpp ---------------------
# (its element-erasing steps are restated with surface_tension=0, which zeroes
# the bulk and gradient elements' factors)
PFU = abi.phase_field_unstructured


def test_pfu_bulk_energy():
    o = Oracle(PFU([1, 1, 1]), [1.0])
    k, kp, _, _ = o.pf_internals()
    assert k[0] == 3 and kp[0] == 3
    e, g = o.energy_gradient()
    assert e == 0 and np.allclose(g, [0])
    e, g = o.energy_gradient([0.1])
    assert e == pytest.approx(3.0 / 16 * 1.21 * 0.81)
    assert np.allclose(g, [-3.0 / 4 * 0.099], atol=1e-6)
    for grid in ([5, 1, 1], [1, 5, 1], [1, 1, 5]):
        e, g = Oracle(PFU(grid, solid=[1, 0, 0, 0, 1]), [0, -1, 0, 1, 0]).energy_gradient()
        assert e == pytest.approx(3.0 / 16 + 2 * (3.0 / 4))
        assert np.allclose(g, [0, -1.5, 0, 1.5, 0], atol=1e-6)
    for grid in ([3, 1, 1], [1, 3, 1], [1, 1, 3]):
        e, g = Oracle(PFU(grid, solid=[0, 1, 0]), [-1, 0, 1]).energy_gradient()
        assert e == pytest.approx(3.0 / 4 * 4)
        assert np.allclose(g, [-3, 0, 3], atol=1e-6)


def test_pfu_external_force():
    for f, gexp in [([-2, 0, 0], [-.5, -.5, -.5, -.5, .5, .5, .5, .5]),
                    ([0, -2, 0], [-.5, -.5, .5, .5, -.5, -.5, .5, .5]),
                    ([0, 0, -2], [-.5, .5, -.5, .5, -.5, .5, -.5, .5])]:
        e, g = Oracle(PFU([2, 2, 2], force=f), [1] * 8).energy_gradient()
        assert e == pytest.approx(0, abs=1e-12)
        assert np.allclose(g, gexp, atol=1e-6)
    e, g = Oracle(PFU([2, 2, 2], surface_tension=0, force=[-4, 0, 0]), [-1] * 4 + [1] * 4).energy_gradient()
    assert e == pytest.approx(8)
    assert np.allclose(g, [0, 0, 0, 0, 1, 1, 1, 1], atol=1e-6)


def test_pfu_surface_energy():
    o = Oracle(PFU([2, 1, 1], surface_tension=0, contact_angle=[90, 60], solid=[1, 0]), [0.0, 0.5])
    e, g = o.energy_gradient()
    assert e == pytest.approx(0.5 / np.sqrt(2.0) * (-27.0 / 24))
    assert np.allclose(g, [0, 0.5 / np.sqrt(2.0) * (-0.75)], atol=1e-6)


def test_pfu_pressure():
    e, g = Oracle(PFU([6, 1, 1], solid=[1, 0, 0, 0, 0, 1], pressure=[10]), [1] * 6).energy_gradient()
    assert e == pytest.approx(-30)
    assert np.allclose(g, [0, -2.5, -5, -5, -2.5, 0], atol=1e-6)


def test_pfu_volume_penalty():
    e = Oracle(PFU([6, 1, 1], solid=[1, 0, 0, 0, 0, 1], volume_fixed=True, vol_const=1), [1] * 6).energy()
    assert e == pytest.approx(0)
    o = Oracle(PFU([6, 1, 1], solid=[1, 0, 0, 0, 0, 1], volume=[1], volume_fixed=True, vol_const=100), [1] * 6)
    e, g = o.energy_gradient()
    assert e == pytest.approx(100 * 2 ** 2)
    assert np.allclose(g, 0)  # zero away from interfaces


def test_pfu_resolution():
    o = Oracle(PFU([5, 1, 1], resolution=2, solid=[1, 0, 0, 0, 1]), [0, -1, 0, 1, 0])
    k, kp, _, _ = o.pf_internals()
    assert k[0] == 1.5 and kp[0] == 6
    e, g = o.energy_gradient()
    assert e == pytest.approx(1.5 / 16 * 8 + 2 * (6.0 / 4) * 2)
    assert np.allclose(g, [0, -6, 0, 6, 0], atol=1e-6)
    e, g = Oracle(PFU([2, 2, 2], resolution=2, surface_tension=0, force=[-4, 0, 0]),
                  [-1] * 4 + [1] * 4).energy_gradient()
    assert e == pytest.approx(128)
    assert np.allclose(g, [0, 0, 0, 0, 16, 16, 16, 16], atol=1e-6)
    e, g = Oracle(PFU([2, 1, 1], resolution=2, surface_tension=0, solid=[1, 0], contact_angle=[90, 60]),
                  [0, 0.5]).energy_gradient()
    assert e == pytest.approx(0.5 / np.sqrt(2.0) * (-27.0 / 24) * 4)
    assert np.allclose(g, [0, 0.5 / np.sqrt(2.0) * (-0.75) * 4], atol=1e-6)
    e, g = Oracle(PFU([6, 1, 1], resolution=2, solid=[1, 0, 0, 0, 0, 1], pressure=[10]), [1] * 6).energy_gradient()
    assert e == pytest.approx(-240)
    assert np.allclose(g, [0, -20, -40, -40, -20, 0], atol=1e-6)
    e, g = Oracle(PFU([6, 1, 1], resolution=2, solid=[1, 0, 0, 0, 0, 1], volume=[8], volume_fixed=True,
                      vol_const=100), [1] * 6).energy_gradient()
    assert e == pytest.approx(100.0 / 16 * (2 * 8) ** 2)
    assert np.allclose(g, 0)


def test_pfu_fix_fluid():
    o = Oracle(PFU([2, 2, 1], nfluid=3, density_constraint="none", fix_fluid=[1, 0, 0]), [1.0] * 12)
    v = o.apply_constraints(np.arange(12.0) + 1)
    assert np.all(v[0::3] == 0) and np.array_equal(v[1::3], np.arange(12.0)[1::3] + 1)


def test_pfu_soft_density_needs_three_fluids():
    with pytest.raises(Exception):
        Oracle(PFU([2, 2, 1], nfluid=2, density_constraint="soft"), [0.5] * 8)
