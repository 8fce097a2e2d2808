"""Generates tests/golden/pillar.npz: the reference's pf-pillar-collapse
benchmark (test/benchmark/pf-pillar-collapse/main.cpp) run with the reference
minim library itself (oracle/_ref/libminim_ref.so; `make -C oracle ref`
first), for the seven contact angles 30..150 at spacing 40.

Per angle: diffuseSolid of the pillar mask (L-BFGS without line search, 100
iterations, fp64), then the critical-pressure bisection, each run L-BFGS
without line search for at most 5000 iterations with fluid 0 fixed and the
hard density constraint.  main.cpp tests for the collapse in a callback at
every iteration and stops the run there; here, as in the GPU test, the test
is on the run's final coordinates (a collapse, once the liquid is at the base,
does not retreat).  The angles run in parallel processes.
Usage: python tests/golden/gen_pillar.py
"""
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)


def _diffuse(ca):
    from minim_gb300 import abi
    from oracle.oracle import Reference
    from tests import workloads as W
    from tests.golden.gen_golden import params_from
    kw = W.pillar_kwargs(ca, diffuse=True)
    r = Reference(params_from("pf", kw), W.pillar_diffuse_init(W.pillar_solid()))
    tol = 1e-8 * kw["surface_tension"][0] * W.PILLAR["res"] ** 2
    res = r.minimise(abi.minimiser("lbfgs", linesearch="none", max_iter=100, tol=tol))
    return r.coords, res.iter


def _run(args):
    ca, p, x0 = args
    from minim_gb300 import abi
    from oracle.oracle import Reference
    from tests import workloads as W
    from tests.golden.gen_golden import params_from
    r = Reference(params_from("pf", W.pillar_kwargs(ca, pressure=p)), x0)
    res = r.minimise(abi.minimiser("lbfgs", linesearch="none", max_iter=5000))
    return W.pillar_failed(r.coords), res.iter


def main():
    from tests import workloads as W
    angles = np.array(W.PILLAR_ANGLES, float)
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(len(angles), os.cpu_count() or 1)) as pool:
        dif = pool.map(_diffuse, angles)
        x0s = [W.pillar_fluid(d) for d, _ in dif]
        lo, hi, hist = W.pillar_bisect(
            lambda idx, p: pool.map(_run, [(angles[i], pi, x0s[i]) for i, pi in zip(idx, p)]),
            len(angles))
    nmax = max(len(h) for h in hist)
    tried = np.full((len(angles), nmax), np.nan)
    failed = np.zeros((len(angles), nmax), np.int8)
    iters = np.zeros((len(angles), nmax), np.int32)
    for a, h in enumerate(hist):
        for k, (p, f, it) in enumerate(h):
            tried[a, k], failed[a, k], iters[a, k] = p, f, it
    d90 = dif[list(angles).index(90)][0]
    np.savez_compressed(
        os.path.join(HERE, "pillar.npz"), angles=angles, lo=lo, hi=hi, tried=tried, failed=failed,
        iters=iters, diffuse_iters=np.array([it for _, it in dif]),
        diffused_sum=np.array([d[0::3].sum() for d, _ in dif]),
        diffused_sq=np.array([(d[0::3] ** 2).sum() for d, _ in dif]),
        diffused90=d90[0::3])
    for a, l, h in zip(angles, lo, hi):
        print(f"{a:5.0f}  critical {0.5 * (l + h):9.2f} +- {0.5 * (h - l):5.2f}   analytic "
              f"{W.pillar_analytic(a):9.2f}")


if __name__ == "__main__":
    main()
