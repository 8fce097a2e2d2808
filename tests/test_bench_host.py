"""Host-side logic of bench.py that needs no GPU: the per-stage FIRE
iteration cost fit recovers known costs from synthetic per-instance
results, and ignores instances that did not reach the iteration limit."""
import types

import numpy as np

import bench
from minim_gb300 import abi


def _results(a32, b32, a64, b64, rng, n=200):
    sizes, res = [], []
    for _ in range(n):
        N = int(rng.integers(13, 401))
        n64 = int(rng.integers(0, 40000))
        it = 100001
        run_us = (a32 * N * N + b32) * (it - n64) + (a64 * N * N + b64) * n64
        sizes.append(N)
        res.append(types.SimpleNamespace(status=abi.RES_MAXITER, iter=it, fp64_iters=n64, run_ms=run_us / 1e3))
    return sizes, res


def test_iteration_cost_fit_recovers_costs():
    rng = np.random.default_rng(3)
    sizes, res = _results(2e-4, 14.0, 1.5e-3, 70.0, rng)
    # converged runs do not enter the fit
    sizes.append(50)
    res.append(types.SimpleNamespace(status=abi.RES_CONVERGED, iter=10, fp64_iters=0, run_ms=1e9))
    f = bench._iteration_cost_fit(sizes, res)
    assert f["instances"] == 200
    assert np.isclose(f["us_per_n2_fp32"], 2e-4, rtol=1e-6)
    assert np.isclose(f["us_fixed_fp32"], 14.0, rtol=1e-6)
    assert np.isclose(f["us_per_n2_fp64"], 1.5e-3, rtol=1e-6)
    assert np.isclose(f["us_fixed_fp64"], 70.0, rtol=1e-6)
    assert np.isclose(f["us_per_iteration_n390"]["fp64"], 1.5e-3 * 390 ** 2 + 70.0)
    assert 0.0 < f["fp64_share_of_instance_time"] < 1.0


def test_iteration_cost_fit_needs_enough_runs():
    rng = np.random.default_rng(4)
    sizes, res = _results(2e-4, 14.0, 1.5e-3, 70.0, rng, n=5)
    assert bench._iteration_cost_fit(sizes, res) is None


def test_oracle_rate_extrapolates_by_stratum():
    """Two strata of small Lennard-Jones clusters, each sampled once and
    standing for 3 and 5 instances: every sampled run converges, so the rate
    is the 8 instances over their extrapolated CPU seconds per thread."""
    from tests.workloads import lj_cluster
    mp = abi.minimiser("lbfgs", m=5, tol=1e-6)
    jobs = {"a": [(abi.lj(), lj_cluster(13, seed=1), None, mp)],
            "b": [(abi.lj(), lj_cluster(20, seed=2), None, mp)]}
    rate, cores, desc = bench._oracle_rate(jobs, {"a": 3, "b": 5})
    assert rate is not None and rate > 0
    assert cores >= 1
    assert "2 instances in 2 strata" in desc and "8 instances" in desc
    # a stratum with no instances contributes nothing; none at all gives no rate
    assert bench._oracle_rate(jobs, {"a": 0, "b": 0})[0] is None
