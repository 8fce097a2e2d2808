"""Per-evaluation parity of the kernels each minimiser stage runs, against the
FP64 oracle at the same point (minim_gpu_eval_kernel through the C ABI).

The minimiser spends almost every iteration in these kernels, not in the
FP64 evaluation behind minim_gpu_energy_gradient: the FP32 stage's
Lennard-Jones tiles (grid team and the batch CTA's symmetric tile path,
energy-only and with gradient), the binary PhaseField quad sweep and the
stepped graph's two-trial line stencil, the general PhaseField sweep, the
BarAndHinge colour scatter, and the FP64 stage's double-float sweeps.  Each
is evaluated once at the workloads' own inputs and sizes (LJ N = 13, 256,
400; PhaseField 192^3 binary and 512^2 ternary with fixed volumes; a 100k
vertex sheet), at the point x and at a trial point x + t p, and compared with
the oracle evaluated at exactly the point the kernel formed (the FP32 paths
round x and p to FP32, as the minimiser's coordinates and directions are).

Tolerances (max |g - g_oracle| / max |g_oracle|; energies relative):
  FP32 stage: gradient 1e-5, energy 2e-6 (FP32 arithmetic per element,
              compensated sums);
  FP64 stage: gradient 2e-7 (double-float arithmetic, the gradient stored in
              FP32 as the minimiser stores it), energy 1e-12.
With MINIM_PARITY_LOG set, the measured errors are appended to that file as
JSON lines.
"""
import json
import os

import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests.workloads import Rng, lj_cluster, pf_noise, pf_simplex, sheet

pytestmark = pytest.mark.gpu

GRAD32, E32 = 1e-5, 2e-6
GRAD64S, E64S = 2e-7, 1e-12

f32 = np.float32


def _log(case, path, **errs):
    fn = os.environ.get("MINIM_PARITY_LOG")
    if fn:
        with open(fn, "a") as f:
            f.write(json.dumps({"case": case, "path": path, **{k: float(v) for k, v in errs.items()}}) + "\n")


def _point32(x, p, t):
    """The point the FP32 paths evaluate: x32 + fl(t32 * p32), in FP32."""
    x32 = np.asarray(x, f32)
    if p is None:
        return x32.astype(np.float64)
    tp = f32(t) * np.asarray(p, f32)
    return (x32 + tp).astype(np.float64)


def _point64s(x, p, t):
    if p is None:
        return np.asarray(x, np.float64)
    return np.asarray(x, np.float64) + t * np.asarray(p, f32).astype(np.float64)


def _errs(e, g, eo, go, escale=None):
    es = max(abs(eo), 1e-300) if escale is None else escale
    de = abs(e - eo) / es
    dg = None if g is None else float(np.max(np.abs(g - go)) / max(np.max(np.abs(go)), 1e-300))
    return de, dg


def _check_paths(case, inst, ora, x, p, t, paths, energy_scale=None):
    """Every path at x (E+g and energy-only) and at x + t p."""
    for path in paths:
        fp32 = path in (abi.EVAL_FP32_GRID, abi.EVAL_FP32_CTA)
        gtol, etol = (GRAD32, E32) if fp32 else (GRAD64S, E64S)
        for pp in (None, p):
            xt = _point32(x, pp, t) if fp32 else _point64s(x, pp, t)
            eo, go = ora.energy_gradient(xt)
            e, g = inst.eval_kernel(path, x, pp, t)
            de, dg = _errs(e, g, eo, go, energy_scale)
            e_only, g_none = inst.eval_kernel(path, x, pp, t, gradient=False)
            de_only, _ = _errs(e_only, None, eo, go, energy_scale)
            _log(case, path, trial=pp is not None, energy_rel_err=de, energy_only_rel_err=de_only,
                 grad_rel_err=dg)
            assert g_none is None
            assert dg <= gtol, (case, path, pp is not None, dg)
            assert de <= etol, (case, path, pp is not None, de, e, eo)
            assert de_only <= etol, (case, path, pp is not None, de_only, e_only, eo)


ALL = (abi.EVAL_FP32_GRID, abi.EVAL_FP32_CTA, abi.EVAL_FP64S_GRID, abi.EVAL_FP64S_CTA)


@pytest.mark.parametrize("n,seed", [(13, 3), (256, 0), (400, 7)])
def test_lj_stage_kernels(n, seed):
    # N = 256 seed 0 is the plain-method cluster; N <= 400 the batched sizes
    p = abi.lj()
    x = lj_cluster(n, seed=seed)
    inst = runtime.Instance(p, x)
    ora = Oracle(p, x)
    _, g0 = ora.energy_gradient(x)
    d = -g0 / max(np.max(np.abs(g0)), 1e-300) * 0.05  # a descent direction of a plausible step
    _check_paths(f"lj{n}", inst, ora, x, d, 0.5, ALL)


def test_lj_stage_kernels_2d_fixed():
    p = abi.lj(ndim=2, sigma=1.1, epsilon=0.7)
    x = lj_cluster(90, seed=11, ndim=2)
    fixed = [0, 1, 7, 100]
    inst = runtime.Instance(p, x, fixed=fixed)
    ora = Oracle(p, x, fixed=fixed)
    d = Rng(5).uniform(x.size) * 0.02 - 0.01
    _check_paths("lj90_2d_fixed", inst, ora, x, d, 1.0, ALL)


def test_pf_binary_192_stage_kernels():
    # the 192^3 binary field of the single-instance workload
    grid = (192, 192, 192)
    p = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0)
    x = pf_noise(grid, seed=0, amp=0.05)
    inst = runtime.Instance(p, x)
    ora = Oracle(p, x)
    _, g0 = ora.energy_gradient(x)
    d = -g0 * 0.1
    _check_paths("pf192", inst, ora, x, d, 1.0, ALL)


@pytest.mark.parametrize("t", [1.0, 0.25])
def test_pf_binary_192_line_stencil(t):
    """The stepped graph's trial pass: two trials (t, t/2) with their
    gradients in one pass, and the energy-only trial."""
    grid = (192, 192, 192)
    p = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0)
    x = pf_noise(grid, seed=0, amp=0.05)
    inst = runtime.Instance(p, x)
    ora = Oracle(p, x)
    _, g0 = ora.energy_gradient(x)
    d = -g0 * 0.1
    e, g, pts = inst.eval_kernel(abi.EVAL_LINES, x, d, t, points=True)
    x32, d32 = np.asarray(x, f32), np.asarray(d, f32)
    for k, tk in enumerate((t, 0.5 * t)):
        # one fused multiply-add per coordinate: the exact x + t p rounded once
        want = (x32.astype(np.float64) + np.float64(f32(tk)) * d32.astype(np.float64)).astype(f32)
        assert np.array_equal(pts[k].astype(f32), want)
        eo, go = ora.energy_gradient(pts[k])
        de, dg = _errs(e[k], g[k], eo, go)
        _log("pf192_lines", abi.EVAL_LINES, trial=k, t=tk, energy_rel_err=de, grad_rel_err=dg)
        assert dg <= GRAD32, (k, dg)
        assert de <= E32, (k, de, e[k], eo)
    e0, _ = inst.eval_kernel(abi.EVAL_LINES, x, d, t, gradient=False)
    eo, _ = ora.energy_gradient(pts[0])
    de0 = abs(e0[0] - eo) / abs(eo)
    _log("pf192_lines_eonly", abi.EVAL_LINES, t=t, energy_rel_err=de0)
    assert de0 <= E32


def test_pf_lines_rejects_general_kernel():
    grid = (8, 8, 8)
    p = abi.phase_field(grid, nfluid=3)
    x = pf_simplex(grid, 3, seed=1)
    inst = runtime.Instance(p, x)
    with pytest.raises(runtime.MinimGpuError) as e:
        inst.eval_kernel(abi.EVAL_LINES, x)
    assert e.value.code == abi.ERR_INVALID


def test_pf_ternary_512_stage_kernels():
    # the largest 2-D three-fluid grid of the batched mixed workload (hard
    # density constraint, fixed volumes)
    grid = (512, 512, 1)
    p = abi.phase_field(grid, nfluid=3, volume_fixed=True)
    x = pf_simplex(grid, 3, seed=5000)
    inst = runtime.Instance(p, x)
    ora = Oracle(p, x)
    _, g0 = ora.energy_gradient(x)
    d = -g0 * 0.05
    _check_paths("pf512_ternary", inst, ora, x, d, 1.0, ALL)


def test_pf_general_terms_stage_kernels():
    # binary field with solid nodes, contact angles, pressure and a body
    # force: the general sweep's optional terms in both stages
    shape = (24, 20, 8)
    solid = np.zeros(shape, np.uint8)
    solid[9:13, 6:10, 2:5] = 1
    solid[:, 0, :] = 1
    ca = Rng(4).uniform(int(np.prod(shape))) * 120 + 30
    x = pf_noise(shape, seed=4, amp=0.9)
    p = abi.phase_field(shape, solid=solid.ravel(), contact_angle=ca, force=[0.1, -0.3, 0.2], pressure=[0.4])
    inst = runtime.Instance(p, x)
    ora = Oracle(p, x)
    d = Rng(5).uniform(x.size) * 0.02 - 0.01
    _check_paths("pf_general_binary", inst, ora, x, d, 1.0, ALL)


@pytest.mark.parametrize("density", ["hard", "soft", "fixed"])
def test_pf_ternary_terms_stage_kernels(density):
    # three fluids with walls, fixed volumes, per-fluid tensions, pressure,
    # body force and confinement under each density constraint
    shape = (40, 36, 1)
    solid = np.zeros(shape, np.uint8)
    solid[:, 0, :] = 1
    x = pf_simplex(shape, 3, seed=5)
    p = abi.phase_field(shape, nfluid=3, solid=solid.ravel(), volume_fixed=True, density_constraint=density,
                        surface_tension=[1.0, 0.8, 1.2], pressure=[0, 0.3, 0],
                        force=[[0, -1, 0], [0.2, 0, 0], [0, 0, 0]], confinement=[0, 1.0, 0])
    inst = runtime.Instance(p, x)
    ora = Oracle(p, x)
    d = Rng(6).uniform(x.size) * 0.02 - 0.01
    _check_paths(f"pf_ternary_{density}", inst, ora, x, d, 1.0, ALL)


def _sheet_oracle(inst, x_flat, pert):
    """The oracle over the instance's own elements (explicit bond and hinge
    lists with their parameters): the triangulation's O(T^2) hinge search is
    out of reach at 100k vertices; the device-built elements are checked
    against the host builder in test_gpu_bah_setup."""
    a = inst.bah_arrays()
    p = abi.bar_and_hinge(bonds=a["bars"], hinges=a["hinges"],
                          rigidity=(a["bar_par"][:, 0].copy(), a["hinge_par"][:, 0].copy()),
                          length0=a["bar_par"][:, 1].copy(), theta0=a["hinge_par"][:, 1].copy())
    return Oracle(p, pert)


@pytest.mark.parametrize("k", [40, 317])
def test_bah_sheet_stage_kernels(k):
    # k = 317: a 100,489-vertex sheet, the largest of the batched workload
    flat, tris, pert = sheet(k, seed=6000 + k)
    inst = runtime.Instance(abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01)), flat)
    inst.coords = pert
    ora = _sheet_oracle(inst, flat, pert)
    _, g0 = ora.energy_gradient(pert)
    d = -g0 / max(np.max(np.abs(g0)), 1e-300) * 0.01
    _check_paths(f"bah{k * k}", inst, ora, pert, d, 1.0, ALL)


def test_stage_eval_rejects_bad_arguments():
    x = lj_cluster(13, seed=1)
    inst = runtime.Instance(abi.lj(), x)
    for path in (-1, 5):
        with pytest.raises(runtime.MinimGpuError) as e:
            inst.eval_kernel(path, x)
        assert e.value.code == abi.ERR_INVALID
    with pytest.raises(runtime.MinimGpuError) as e:
        inst.eval_kernel(abi.EVAL_FP32_GRID, x, points=True)
    assert e.value.code == abi.ERR_INVALID


@pytest.mark.parametrize("grid", [(192, 192, 192), (5, 12, 64), (16, 8, 32), (6, 16, 256)])
def test_pf_line_stencil_tma(grid):
    """The two-trial line stencil with its lines staged through tensor-map
    tiles: points and gradients bitwise those of the direct stencil (same
    arithmetic per quad), energies those of the direct stencil up to the
    order of the sums, and both trials within the FP32 tolerances of the
    oracle.  The small grids put every strip at the periodic boundary in y
    (one-line wrap copies) and give plane runs of one to three planes."""
    p = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0)
    x = pf_noise(grid, seed=3, amp=0.05)
    inst = runtime.Instance(p, x)
    ora = Oracle(p, x)
    _, g0 = ora.energy_gradient(x)
    d = -g0 * 0.1
    for t in (1.0, 0.25):
        e, g, pts = inst.eval_kernel(abi.EVAL_LINES_TMA, x, d, t, points=True)
        ed, gd, ptd = inst.eval_kernel(abi.EVAL_LINES, x, d, t, points=True)
        assert np.array_equal(pts, ptd)
        assert np.array_equal(g, gd)
        for k in range(2):
            assert abs(e[k] - ed[k]) <= 1e-12 * abs(ed[k]), (k, e[k], ed[k])
            eo, go = ora.energy_gradient(pts[k])
            de, dg = _errs(e[k], g[k], eo, go)
            _log("pf_lines_tma_%dx%dx%d" % grid, abi.EVAL_LINES_TMA, trial=k, t=t, energy_rel_err=de,
                 grad_rel_err=dg)
            assert dg <= GRAD32, (k, dg)
            assert de <= E32, (k, de)


def test_pf_line_stencil_tma_rejects_grids():
    for grid in [(8, 8, 36), (8, 6, 32), (8, 4, 32), (2, 8, 32)]:
        p = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0)
        x = pf_noise(grid, seed=1, amp=0.05)
        inst = runtime.Instance(p, x)
        with pytest.raises(runtime.MinimGpuError) as e:
            inst.eval_kernel(abi.EVAL_LINES_TMA, x, np.zeros_like(x), 1.0)
        assert e.value.code == abi.ERR_INVALID
