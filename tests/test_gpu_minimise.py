"""Minimisation parity on the GPU (single-instance grid path and batched
path) against the FP64 oracle.

Parity protocol (LJ landscapes are chaotic, so trajectories may part):
  * the returned point is a minimum under the oracle: FP64 RMS(g) < tol;
  * the returned energy equals the oracle's energy at that point to 1e-8
    relative (absolute floor 1e-8 * max(|E|, |E_init|) near zero);
  * for the reference's known-answer cases (BarAndHinge hinge minima) the
    coordinates match the analytic minima to 1e-4, as the reference test does;
  * in FP64 mode small cases follow the oracle to the same minimum.
"""
import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests.workloads import lj_cluster, pf_noise, pf_simplex, sheet

pytestmark = pytest.mark.gpu


def check_minimum(p, x0, x, res, tol, fixed=None, gd=False):
    """gd: GradDescent tests convergence on the gradient before its last
    step (src/minimisers/GradDescent.cpp:27-46), so the returned point is one
    step further.  Armijo accepts steps that overshoot along stiff pair modes
    (up to a reflection), so that step can raise the gradient a few times
    over tol; the bound used is 10 tol."""
    ora = Oracle(p, x0, fixed=fixed)
    e, g = ora.energy_gradient(x)
    e_init = ora.energy(x0)
    floor = 1e-8 * max(abs(e), abs(e_init))
    if not gd:
        assert abs(res.energy - e) <= max(1e-8 * abs(e), floor), (res.energy, e)
    rms = np.sqrt(np.mean(g ** 2))
    assert rms < (10 * tol if gd else tol), rms
    return e


@pytest.mark.parametrize("seed", [3, 5, 21, 42, 77])
def test_lj_grid_mixed_seeds(seed):
    """Mixed precision must leave the FP32 stage on its own for any start
    (the line search stops resolving the decrease near the FP32 floor)."""
    x0 = lj_cluster(13, seed=seed)
    p = abi.lj()
    inst = runtime.Instance(p, x0)
    r = inst.minimise(abi.minimiser("lbfgs", tol=1e-6, max_iter=20000))
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    check_minimum(p, x0, inst.coords, r, 1e-6)


@pytest.mark.parametrize("method,ls", [("lbfgs", None), ("fire", "backtracking"), ("gd", None)])
@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_lj_grid_path(method, ls, prec):
    x0 = lj_cluster(13, seed=11)
    p = abi.lj()
    inst = runtime.Instance(p, x0)
    tol = 1e-6 if method != "gd" else 1e-5
    mp = abi.minimiser(method, linesearch=ls, tol=tol, precision=prec, max_iter=200000)
    r = inst.minimise(mp)
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    check_minimum(p, x0, inst.coords, r, tol, gd=(method == "gd"))


def test_lj_fp64_follows_oracle():
    x0 = lj_cluster(20, seed=12)
    p = abi.lj()
    mp = abi.minimiser("lbfgs", tol=1e-6, precision="fp64")
    inst = runtime.Instance(p, x0)
    r = inst.minimise(mp)
    ora = Oracle(p, x0)
    ro = ora.minimise(mp)
    assert r.status == abi.RES_CONVERGED
    assert abs(r.energy - ro.energy) <= 1e-8 * abs(ro.energy)
    assert np.max(np.abs(inst.coords - ora.coords)) < 1e-4


def test_fire_first_step():
    # Fire().setMaxIter(0): one iteration from v = 0 moves x by -dt^2/2 * g
    # with dt = dtMax = 0.1/sqrt(|g|) (reference test/unit/Fire_test.cpp:25-40)
    x0 = lj_cluster(8, seed=13)
    p = abi.lj()
    mp = abi.minimiser("fire", linesearch="backtracking", max_iter=0, precision="fp64")
    inst = runtime.Instance(p, x0)
    g = inst.gradient()
    inst.minimise(mp)
    dt = 0.1 / np.sqrt(np.linalg.norm(g))
    step = -0.5 * dt * dt * g
    # FP64 coordinates; the velocity and step vectors are stored in FP32
    assert np.max(np.abs(inst.coords - x0 - step)) <= 1e-6 * np.max(np.abs(step))


@pytest.mark.parametrize("target,expected", [
    (1e-6, "a"), (np.pi / 2, "b"), (np.pi, "c"), (3 * np.pi / 2, "d"), (2 * np.pi - 1e-6, "e")])
@pytest.mark.parametrize("path", ["grid", "batch"])
def test_bah_hinge_minima(target, expected, path):
    # reference test/unit/BarAndHinge_test.cpp:13-56
    s2 = np.sqrt(2)
    dz = s2 / 2
    exp = {
        "a": [0, 0, 0.5 + dz, 0, -s2, 0.5 - dz, 0, s2, 0.5 - dz, 0, 0, 0.5 + dz],
        "b": [-1, 0, 1, 0, -s2, 0, 0, s2, 0, 1, 0, 1],
        "c": [-s2, 0, 0.5, 0, -s2, 0.5, 0, s2, 0.5, s2, 0, 0.5],
        "d": [-1, 0, 0, 0, -s2, 1, 0, s2, 1, 1, 0, 0],
        "e": [0, 0, 0.5 - dz, 0, -s2, 0.5 + dz, 0, s2, 0.5 + dz, 0, 0, 0.5 - dz],
    }[expected]
    x0 = np.array([-1, 0, 1, 0, -s2, 0, 0, s2, 0, 1, 0, 1.0])
    p = abi.bar_and_hinge(triangulation=[[0, 1, 2], [1, 3, 2]], rigidity=(100, 1), theta0=[target])
    inst = runtime.Instance(p, x0)
    # The two folded targets sit on the knife edge of the reference's
    # dihedral wrap (theta jumps between 0 and 2*pi where n1.b3 changes
    # sign); following the reference's path onto the same side of the fold
    # needs FP64 coordinates throughout.
    mp = abi.minimiser("lbfgs", precision="fp64")
    if path == "grid":
        r = inst.minimise(mp)
    else:
        b = runtime.Batch()
        b.add(inst, mp)
        r = b.run()[0]
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    assert np.allclose(inst.coords, exp, atol=1e-4), inst.coords


@pytest.mark.parametrize("target", [1e-6, 2 * np.pi - 1e-6])
def test_bah_fold_mixed_precision_is_a_minimum(target):
    """In mixed precision the fold may be reached from the other side; the
    result must still be a minimum of the reference's energy (E ~ 0)."""
    s2 = np.sqrt(2)
    x0 = np.array([-1, 0, 1, 0, -s2, 0, 0, s2, 0, 1, 0, 1.0])
    p = abi.bar_and_hinge(triangulation=[[0, 1, 2], [1, 3, 2]], rigidity=(100, 1), theta0=[target])
    inst = runtime.Instance(p, x0)
    r = inst.minimise(abi.minimiser("lbfgs"))
    assert r.status == abi.RES_CONVERGED
    check_minimum(p, x0, inst.coords, r, 1e-6)
    assert r.energy < 1e-10


def test_batch_lj_mixed_methods():
    p = abi.lj()
    insts, x0s, mps = [], [], []
    for i, n in enumerate([13, 38, 55, 13, 100, 7, 150, 26]):
        x0 = lj_cluster(n, seed=100 + i)
        meth = ["lbfgs", "fire", "gd", "lbfgs"][i % 4]
        mp = abi.minimiser(meth, linesearch="backtracking" if meth == "fire" else None,
                           dt_max=0.0, tol=1e-6 if meth != "gd" else 1e-5, max_iter=200000)
        insts.append(runtime.Instance(p, x0))
        x0s.append(x0)
        mps.append(mp)
    b = runtime.Batch()
    for inst, mp in zip(insts, mps):
        b.add(inst, mp)
    res = b.run()
    for inst, x0, mp, r in zip(insts, x0s, mps, res):
        assert r.status == abi.RES_CONVERGED, r.as_dict()
        check_minimum(p, x0, inst.coords, r, mp.tol, gd=(mp.method == abi.GD))


def test_batch_alone_equals_mixed():
    p = abi.lj()
    x0 = lj_cluster(40, seed=200)
    mp = abi.minimiser("lbfgs", tol=1e-6)
    a = runtime.Instance(p, x0)
    ba = runtime.Batch()
    ba.add(a, mp)
    ra = ba.run(threads=128)[0]
    others = [runtime.Instance(p, lj_cluster(n, seed=300 + n)) for n in (13, 80, 120, 33)]
    b = runtime.Instance(p, x0)
    bb = runtime.Batch()
    for o in others[:2]:
        bb.add(o, mp)
    bb.add(b, mp)
    for o in others[2:]:
        bb.add(o, mp)
    rb = bb.run(threads=128)[2]
    assert ra.iter == rb.iter and ra.energy == rb.energy
    assert np.array_equal(a.coords, b.coords)


def test_pf_binary_minimise():
    grid = (12, 12, 12)
    x0 = pf_noise(grid, seed=21)
    p = abi.phase_field(grid)
    inst = runtime.Instance(p, x0)
    mp = abi.minimiser("lbfgs", m=10, tol=1e-7)
    r = inst.minimise(mp)
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    check_minimum(p, x0, inst.coords, r, 1e-7)


@pytest.mark.parametrize("grid,prec", [((64, 64, 64), "mixed"), ((64, 64, 66), "mixed"), ((64, 64, 64), "fp32")])
def test_pf_binary_minimise_stepped(grid, prec):
    """Large binary PhaseField: the FP32 stage runs as a graph of phase
    kernels (quad stencil when nz % 4 == 0, scalar stencil otherwise); the
    result is a minimum under the oracle, like the persistent path's."""
    x0 = pf_noise(grid, seed=23, amp=0.05)
    p = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0)
    inst = runtime.Instance(p, x0)
    tol = 1e-7 if prec == "mixed" else 1e-5
    r = inst.minimise(abi.minimiser("lbfgs", m=10, tol=tol, precision=prec))
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    st = runtime.last_run_stats()
    assert st["launches"] > 20  # phase kernels, not one persistent launch per slice
    check_minimum(p, x0, inst.coords, r, tol)


def test_pf_stepped_max_iter():
    """The stepped path stops at max_iter like the persistent one."""
    grid = (64, 64, 64)
    x0 = pf_noise(grid, seed=25, amp=0.05)
    inst = runtime.Instance(abi.phase_field(grid, interface_size=1.0, surface_tension=1.0), x0)
    r = inst.minimise(abi.minimiser("lbfgs", m=10, tol=1e-7, max_iter=19))
    assert r.status == abi.RES_MAXITER, r.as_dict()
    assert r.iter == 20


@pytest.mark.parametrize("switch", ["MINIM_GPU_STEPPED", "MINIM_GPU_TRIAL_PAIRS"])
def test_pf_stepped_matches_persistent_path(switch):
    """Same minimisation with the stepped FP32 stage switched off, or with
    one line-search trial per pass instead of two (separate process): same
    minimum to the tolerance, similar iteration count."""
    import json
    import os
    import subprocess
    import sys
    grid = (64, 64, 64)
    x0 = pf_noise(grid, seed=24, amp=0.05)
    p = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0)
    inst = runtime.Instance(p, x0)
    r = inst.minimise(abi.minimiser("lbfgs", m=10, tol=1e-7))
    code = (
        "import json, sys; sys.path.insert(0, '.');"
        "from minim_gb300 import abi, runtime; from tests.workloads import pf_noise;"
        "g = (64, 64, 64); x0 = pf_noise(g, seed=24, amp=0.05);"
        "i = runtime.Instance(abi.phase_field(g, interface_size=1.0, surface_tension=1.0), x0);"
        "r = i.minimise(abi.minimiser('lbfgs', m=10, tol=1e-7));"
        "print(json.dumps({'status': r.status, 'iter': r.iter, 'energy': r.energy}))"
    )
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, **{switch: "0"})
    out = subprocess.run([sys.executable, "-c", code], cwd=repo, env=env, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    q = json.loads(out.stdout.strip().splitlines()[-1])
    assert r.status == q["status"] == abi.RES_CONVERGED
    e_init = Oracle(p, x0).energy(x0)
    assert abs(r.energy - q["energy"]) <= 1e-8 * max(abs(r.energy), abs(e_init))
    assert abs(r.iter - q["iter"]) <= 0.2 * q["iter"] + 10


@pytest.mark.parametrize("extra", [{"max_step": 50.0}, {"linesearch": "none"}])
def test_pf_stepped_options_match_persistent_path(extra):
    """A step cap (the one-trial graph with pass B's set-up) and no line
    search (the two-trial graph's gradient-only passes) against the
    persistent kernel (separate process)."""
    import json
    import os
    import subprocess
    import sys
    grid = (64, 64, 64)
    x0 = pf_noise(grid, seed=28, amp=0.05)
    p = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0)
    kw = dict(m=10, tol=1e-7, max_iter=20000, **extra)
    r = runtime.Instance(p, x0).minimise(abi.minimiser("lbfgs", **kw))
    code = (
        "import json, sys; sys.path.insert(0, '.');"
        "from minim_gb300 import abi, runtime; from tests.workloads import pf_noise;"
        "g = (64, 64, 64); x0 = pf_noise(g, seed=28, amp=0.05);"
        "i = runtime.Instance(abi.phase_field(g, interface_size=1.0, surface_tension=1.0), x0);"
        f"r = i.minimise(abi.minimiser('lbfgs', **{kw!r}));"
        "print(json.dumps({'status': r.status, 'iter': r.iter, 'energy': r.energy}))"
    )
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-c", code], cwd=repo, env=dict(os.environ, MINIM_GPU_STEPPED="0"),
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    q = json.loads(out.stdout.strip().splitlines()[-1])
    assert r.status == q["status"] == abi.RES_CONVERGED, (r.as_dict(), q)
    e_init = Oracle(p, x0).energy(x0)
    assert abs(r.energy - q["energy"]) <= 1e-8 * max(abs(r.energy), abs(e_init))
    assert abs(r.iter - q["iter"]) <= 0.2 * q["iter"] + 10


def test_pf_stepped_graph_reuse():
    """Instances of one shape share the cached stepped graph: the same input
    gives bitwise the same result before and after another instance ran."""
    grid = (64, 64, 64)
    p = abi.phase_field(grid, interface_size=1.0, surface_tension=1.0)
    mp = abi.minimiser("lbfgs", m=10, tol=1e-7)
    x0, x1 = pf_noise(grid, seed=26, amp=0.05), pf_noise(grid, seed=27, amp=0.05)
    runs = []
    for x in (x0, x1, x0):
        inst = runtime.Instance(p, x)
        r = inst.minimise(mp)
        assert r.status == abi.RES_CONVERGED, r.as_dict()
        runs.append((r.iter, r.evals, r.energy, inst.coords))
        inst.close()
    assert runs[0][:3] == runs[2][:3]
    assert np.array_equal(runs[0][3], runs[2][3])
    assert runs[1][2] != runs[0][2]


def test_pf_ternary_volume_minimise_batch():
    shape = (24, 24, 1)
    p = abi.phase_field(shape, nfluid=3, volume_fixed=True)
    x0 = pf_simplex(shape, 3, seed=22)
    inst = runtime.Instance(p, x0)
    mp = abi.minimiser("lbfgs", tol=1e-7, max_iter=20000)
    b = runtime.Batch()
    b.add(inst, mp)
    r = b.run()[0]
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    x = inst.coords
    check_minimum(p, x0, x, r, 1e-7)
    # the projection keeps each fluid's volume and the per-node density
    v0 = x0.reshape(-1, 3).sum(axis=0)
    v1 = x.reshape(-1, 3).sum(axis=0)
    assert np.allclose(v0, v1, rtol=0, atol=1e-6 * x0.size)
    assert np.allclose(x.reshape(-1, 3).sum(axis=1), 1.0, atol=1e-6)


def test_bah_sheet_minimise_batch():
    flat, tris, pert = sheet(10, seed=23)
    p = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01))
    inst = runtime.Instance(p, flat)
    inst.coords = pert
    mp = abi.minimiser("lbfgs", tol=1e-7)
    b = runtime.Batch()
    b.add(inst, mp)
    r = b.run()[0]
    assert r.status == abi.RES_CONVERGED, r.as_dict()
    ora = Oracle(p, flat)
    e, g = ora.energy_gradient(inst.coords)
    assert np.sqrt(np.mean(g ** 2)) < 1e-7
    assert abs(r.energy - e) <= 1e-8 * max(abs(e), abs(ora.energy(pert)))


def test_server_roundtrip():
    p = abi.lj()
    srv = runtime.Server(slice_iters=32)
    ids = {}
    for i, n in enumerate([13, 30, 60, 13, 90]):
        x0 = lj_cluster(n, seed=400 + i)
        ids[srv.submit(p, x0, abi.minimiser("lbfgs", tol=1e-6))] = x0
    done = {}
    for _ in range(10000):
        srv.step()
        for rid, r in srv.poll():
            done[rid] = r
        if len(done) == len(ids):
            break
    assert len(done) == len(ids)
    for rid, r in done.items():
        assert r.status == abi.RES_CONVERGED
        assert r.latency_ms > 0
        x = srv.take(rid)
        check_minimum(p, ids[rid], x, r, 1e-6)


@pytest.mark.parametrize("amp", [1e-4, 0.0])
def test_mixed_start_near_convergence_runs_fp64(amp):
    """A start within 100x of the tolerance (a sheet at its rest shape, or
    barely perturbed from it) is minimised in FP64 from the exact start:
    rounding it to FP32 would add noise that the FP64 stage must then relax
    through the soft hinge modes.  Mixed precision then takes about as many
    iterations as FP64."""
    from tests.workloads import Rng
    flat, tris, _ = sheet(48, seed=6100)
    x0 = flat.copy()
    x0[2::3] += Rng(6101).normal(48 * 48) * amp
    p = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01))
    out = {}
    for prec in ("fp64", "mixed"):
        inst = runtime.Instance(p, flat)
        inst.coords = x0
        b = runtime.Batch()
        b.add(inst, abi.minimiser("lbfgs", tol=1e-7, precision=prec, max_iter=50000))
        r = b.run()[0]
        assert r.status == abi.RES_CONVERGED, (prec, r.as_dict())
        ora = Oracle(p, flat)
        e, g = ora.energy_gradient(inst.coords)
        assert np.sqrt(np.mean(g ** 2)) < 1e-7
        out[prec] = r
    # the whole run in FP64 coordinates (double-float arithmetic in mixed
    # mode, so the iteration counts differ by rounding, not by the FP32
    # noise relaxation that took thousands of iterations)
    info = {k: v.as_dict() for k, v in out.items()}
    assert out["mixed"].fp64_iters >= out["mixed"].iter, info
    assert out["mixed"].iter <= 1.5 * out["fp64"].iter + 10, info
