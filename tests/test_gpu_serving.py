"""Continuous batching and failure handling on the GPU (through the C ABI).

* A request's result does not depend on what else the server is running:
  PhaseField, BarAndHinge and Lennard-Jones requests submitted at staggered
  steps into a running server, each crossing many slices, end bitwise equal
  to the same request run alone through a server.
* Failure paths, with every failure made on the host or by a bounded wait
  that nothing releases (no GPU fault): a NaN-poisoned instance in a batch
  ends with status NAN and leaves its neighbours bit-identical to a clean
  run; admission rejects a request whose workspace exceeds the memory
  budget; cancelling a resident request frees its slot between steps and
  leaves the others' results unchanged; the device barrier's bounded wait
  gives up with an error the host reads, and the GPU keeps working.
"""
import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests.workloads import lj_cluster, pf_noise, sheet

pytestmark = pytest.mark.gpu

SLICE = 16


def _requests():
    grid = (48, 40, 1)
    flat, tris, pert = sheet(20, seed=61)
    p0 = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01))
    _, bpar, _, hpar = runtime.bah_elements(p0, flat)
    pbah = abi.bar_and_hinge(triangulation=tris, rigidity=(1, 0.01), length0=bpar[:, 1].copy(),
                             theta0=hpar[:, 1].copy())
    return {
        "lj40": (abi.lj(), lj_cluster(40, seed=71), abi.minimiser("lbfgs", m=5, tol=1e-6)),
        "pf": (abi.phase_field(grid, interface_size=1.0, surface_tension=1.0), pf_noise(grid, seed=72),
               abi.minimiser("lbfgs", m=5, tol=1e-7)),
        "bah": (pbah, pert, abi.minimiser("lbfgs", m=5, tol=1e-7)),
        "lj150": (abi.lj(), lj_cluster(150, seed=73), abi.minimiser("lbfgs", m=5, tol=1e-6)),
        "fire60": (abi.lj(), lj_cluster(60, seed=74),
                   abi.minimiser("fire", linesearch="backtracking", dt_max=0.0, tol=1e-6)),
    }


def _drain(srv, want, on_step=None, max_steps=100000):
    done = {}
    for step in range(max_steps):
        if on_step:
            on_step(step)
        srv.step()
        for rid, r in srv.poll():
            done[rid] = r
        if all(w in done for w in want()):
            return done, step
    raise AssertionError("server did not finish")


def _alone(p, x0, mp):
    srv = runtime.Server(slice_iters=SLICE)
    rid = srv.submit(p, x0, mp)
    done, steps = _drain(srv, lambda: [rid])
    r = done[rid]
    x = srv.take(rid)
    srv.close()
    return r, x, steps


def test_server_request_same_alone_and_in_mix():
    reqs = _requests()
    alone = {k: _alone(*v) for k, v in reqs.items()}
    for k, (r, _, steps) in alone.items():
        assert r.status == abi.RES_CONVERGED, (k, r.as_dict())
    # every request crosses slice boundaries
    assert all(steps >= 3 for _, _, steps in alone.values()), {k: v[2] for k, v in alone.items()}
    # staggered arrival into a running server, with filler requests around
    srv = runtime.Server(slice_iters=SLICE)
    arrive = {0: ["lj150"], 2: ["pf"], 3: ["fire60"], 5: ["bah"], 7: ["lj40"]}
    ids = {}
    fillers = []

    def on_step(step):
        for k in arrive.get(step, []):
            ids[k] = srv.submit(*reqs[k])
        if step in (1, 4, 6):
            fillers.append(srv.submit(abi.lj(), lj_cluster(90 + step, seed=800 + step),
                                      abi.minimiser("lbfgs", m=5, tol=1e-6)))
            g = (32 + step, 36, 1)
            fillers.append(srv.submit(abi.phase_field(g), pf_noise(g, seed=810 + step),
                                      abi.minimiser("lbfgs", m=5, tol=1e-7)))

    done, _ = _drain(srv, lambda: list(ids.values()) + fillers if len(ids) == len(reqs) else [-1],
                     on_step=on_step)
    for k, rid in ids.items():
        ra, xa, _ = alone[k]
        rm = done[rid]
        xm = srv.take(rid)
        assert rm.status == ra.status, k
        assert (rm.iter, rm.evals, rm.fp64_iters) == (ra.iter, ra.evals, ra.fp64_iters), k
        assert rm.energy == ra.energy, k
        assert np.array_equal(xm, xa), k
    srv.close()


def test_batch_alone_equals_mixed_tuned_shapes():
    """Default (autotuned) launch shapes depend on an instance's own key, so
    a cluster gives the same result alone and next to much larger ones."""
    p = abi.lj()
    mp = abi.minimiser("lbfgs", tol=1e-6)
    x0 = lj_cluster(40, seed=210)
    a = runtime.Instance(p, x0)
    ba = runtime.Batch()
    ba.add(a, mp)
    ra = ba.run()[0]
    b = runtime.Instance(p, x0)
    bb = runtime.Batch()
    others = [runtime.Instance(p, lj_cluster(n, seed=220 + n)) for n in (300, 13, 200)]
    bb.add(others[0], mp)
    bb.add(b, mp)
    for o in others[1:]:
        bb.add(o, mp)
    rb = bb.run()[1]
    assert ra.status == abi.RES_CONVERGED
    assert (ra.iter, ra.evals, ra.energy) == (rb.iter, rb.evals, rb.energy)
    assert np.array_equal(a.coords, b.coords)


def test_nan_instance_leaves_batch_neighbours_unchanged():
    p = abi.lj()
    mp = abi.minimiser("lbfgs", tol=1e-6)
    xs = [lj_cluster(n, seed=500 + n) for n in (20, 45, 70)]
    bad = lj_cluster(45, seed=599)
    bad[7] = np.nan

    def run(include_bad):
        insts = [runtime.Instance(p, x) for x in xs]
        b = runtime.Batch()
        b.add(insts[0], mp)
        if include_bad:
            ib = runtime.Instance(p, bad)
            b.add(ib, mp)
        b.add(insts[1], mp)
        b.add(insts[2], mp)
        res = b.run()
        if include_bad:
            rbad = res.pop(1)
            return res, [i.coords for i in insts], rbad
        return res, [i.coords for i in insts], None

    clean, xc, _ = run(False)
    mixed, xm, rbad = run(True)
    assert rbad.status == abi.RES_NAN, rbad.as_dict()
    for rc, rm, a, b in zip(clean, mixed, xc, xm):
        assert rc.status == abi.RES_CONVERGED
        assert (rc.iter, rc.energy) == (rm.iter, rm.energy)
        assert np.array_equal(a, b)


def test_nan_single_instance_status():
    x = lj_cluster(30, seed=3)
    x[4] = np.inf
    inst = runtime.Instance(abi.lj(), x)
    r = inst.minimise(abi.minimiser("lbfgs", tol=1e-6))
    assert r.status == abi.RES_NAN


def test_server_rejects_by_memory_budget():
    srv = runtime.Server(max_bytes=64 << 10, slice_iters=SLICE)
    grid = (64, 64, 64)
    big = srv.submit(abi.phase_field(grid), pf_noise(grid, seed=9), abi.minimiser("lbfgs", tol=1e-7))
    x0 = lj_cluster(13, seed=9)
    small = srv.submit(abi.lj(), x0, abi.minimiser("lbfgs", tol=1e-6))
    done, _ = _drain(srv, lambda: [big, small])
    assert done[big].status == abi.RES_REJECTED
    assert done[small].status == abi.RES_CONVERGED
    x = srv.take(small)
    e, g = Oracle(abi.lj(), x0).energy_gradient(x)
    assert np.sqrt(np.mean(g ** 2)) < 1e-6
    # a rejected request's coordinates are its start
    assert np.array_equal(srv.take(big), pf_noise(grid, seed=9))
    srv.close()


def test_server_cancel_resident_request():
    reqs = _requests()
    ra, xa, _ = _alone(*reqs["lj150"])
    srv = runtime.Server(slice_iters=SLICE)
    grid = (40, 40, 40)
    long_id = srv.submit(abi.phase_field(grid), pf_noise(grid, seed=31), abi.minimiser("lbfgs", tol=1e-9))
    assert srv.step()[0] == 1
    other = srv.submit(*reqs["lj150"])
    assert srv.step()[0] == 2
    srv.cancel(long_id)
    done, _ = _drain(srv, lambda: [long_id, other])
    assert done[long_id].status == abi.RES_CANCELLED
    # the other request ran next to the cancelled one, then alone: the same
    # result as alone throughout
    rm = done[other]
    assert (rm.status, rm.iter, rm.energy) == (ra.status, ra.iter, ra.energy)
    assert np.array_equal(srv.take(other), xa)
    srv.close()


def test_bounded_wait_gives_up_and_gpu_stays_usable():
    timed_out, ms = runtime.wait_probe(50)
    assert timed_out
    assert 40.0 <= ms < 5000.0, ms
    with pytest.raises(runtime.MinimGpuError) as e:
        runtime.wait_probe(0)
    assert e.value.code == abi.ERR_INVALID
    # the context is intact: a minimisation afterwards converges
    x0 = lj_cluster(13, seed=5)
    inst = runtime.Instance(abi.lj(), x0)
    r = inst.minimise(abi.minimiser("lbfgs", tol=1e-6))
    assert r.status == abi.RES_CONVERGED
