"""The batch launch-shape autotuner (threads per CTA per potential kind, size
bucket, method and precision), through the C ABI: every candidate is timed
on the batch's own instances the first time a key is seen, the choice is
reported, every candidate shape gives a minimum under the oracle, and a
cache file carries the choices to another process."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from minim_gb300 import abi, runtime
from oracle.oracle import Oracle
from tests.workloads import lj_cluster, pf_simplex

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_tuner_measures_every_candidate():
    p = abi.lj()
    mp = abi.minimiser("lbfgs", m=5, tol=1e-6)
    b = runtime.Batch()
    insts = [runtime.Instance(p, lj_cluster(n, seed=900 + n)) for n in (330, 340, 350)]
    for i in insts:
        b.add(i, mp)
    b.run()
    rows = [r for r in runtime.tune_table() if r["kind"] == "lj" and r["method"] == abi.LBFGS]
    assert rows, runtime.tune_table()
    for r in rows:
        assert r["threads"] in (64, 128, 256)
        if not r["measured"]:
            continue
        ms = r["candidate_ms"]
        assert all(t > 0 for t in ms)
        if r["bucket"] < 8:
            # one CTA of 64 / 128 / 256 threads: the fastest is taken
            assert len(ms) == 3 and r["ctas"] == 1
            assert min(ms) == ms[(64, 128, 256).index(r["threads"])]
        else:
            # above 512 particles also clusters of 2 / 4 / 8 CTAs (timed on
            # the largest instance), then the one-CTA time of that instance
            assert len(ms) == 7 and r["ctas"] in (1, 2, 4, 8)


@pytest.mark.parametrize("threads", [64, 128, 256])
def test_every_lj_candidate_gives_a_minimum(threads):
    p = abi.lj()
    x0 = lj_cluster(120, seed=950)
    inst = runtime.Instance(p, x0)
    b = runtime.Batch()
    b.add(inst, abi.minimiser("lbfgs", m=5, tol=1e-6))
    r = b.run(threads=threads)[0]
    assert r.status == abi.RES_CONVERGED
    e, g = Oracle(p, x0).energy_gradient(inst.coords)
    assert np.sqrt(np.mean(g ** 2)) < 1e-6
    assert abs(r.energy - e) <= 1e-8 * abs(e)


@pytest.mark.parametrize("threads", [256, 512])
def test_every_grid_candidate_gives_a_minimum(threads):
    grid = (48, 48, 1)
    p = abi.phase_field(grid, nfluid=3, volume_fixed=True)
    x0 = pf_simplex(grid, 3, seed=951)
    inst = runtime.Instance(p, x0)
    b = runtime.Batch()
    b.add(inst, abi.minimiser("lbfgs", tol=1e-7, max_iter=20000))
    r = b.run(threads=threads)[0]
    assert r.status == abi.RES_CONVERGED
    ora = Oracle(p, x0)
    e, g = ora.energy_gradient(inst.coords)
    assert np.sqrt(np.mean(g ** 2)) < 1e-7
    assert abs(r.energy - e) <= 1e-8 * max(abs(e), abs(ora.energy(x0)))


_CHILD = r"""
import json, sys
sys.path.insert(0, sys.argv[1])
from minim_gb300 import abi, runtime
from tests.workloads import lj_cluster
b = runtime.Batch()
insts = [runtime.Instance(abi.lj(), lj_cluster(n, seed=n)) for n in (70, 80)]
for i in insts:
    b.add(i, abi.minimiser("fire", dt_max=0.1, tol=1e-6, max_iter=300))
b.run()
print(json.dumps(runtime.tune_table()))
"""


def test_tune_cache_file_across_processes(tmp_path):
    cache = str(tmp_path / "tune.txt")
    env = dict(os.environ, MINIM_GPU_TUNE_CACHE=cache)
    outs = []
    for _ in range(2):
        r = subprocess.run([sys.executable, "-c", _CHILD, REPO], capture_output=True, text=True, env=env,
                           timeout=300)
        assert r.returncode == 0, r.stderr
        outs.append(json.loads(r.stdout.strip().splitlines()[-1]))
    first = [t for t in outs[0] if t["kind"] == "lj"]
    second = [t for t in outs[1] if t["kind"] == "lj"]
    assert first and all(t["measured"] for t in first)
    assert second and not any(t["measured"] for t in second)
    assert [t["threads"] for t in first] == [t["threads"] for t in second]
    assert os.path.getsize(cache) > 0


def test_tuning_off_takes_the_size_rule(tmp_path):
    env = dict(os.environ, MINIM_GPU_TUNE="0")
    r = subprocess.run([sys.executable, "-c", _CHILD, REPO], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr
    assert json.loads(r.stdout.strip().splitlines()[-1]) == []
