"""Instance sharding over 2 ranks (gloo, CPU): every instance is minimised
exactly once, by one rank, and the gathered results equal a single-rank run.
The per-rank worker is the FP64 oracle (no GPU here)."""
import os

import numpy as np
import torch.multiprocessing as mp

from minim_gb300 import shard

SIZES = [13, 7, 26, 19, 38, 8, 13, 30]


def test_partition_balanced_and_complete():
    costs = [float(n) ** 2 for n in SIZES]
    parts = shard.partition(costs, 2)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(SIZES)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)
    assert shard.partition(costs, 1) == [list(range(len(SIZES)))]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from minim_gb300 import abi
    from oracle.oracle import Oracle
    from tests.workloads import lj_cluster
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    costs = [shard.instance_cost(0, 3 * n) for n in SIZES]
    mine = shard.partition(costs, world)[rank]
    local = []
    for i in mine:
        o = Oracle(abi.lj(), lj_cluster(SIZES[i], seed=i))
        r = o.minimise(abi.minimiser("lbfgs", tol=1e-6))
        local.append((r.energy, r.iter, o.coords.tolist()))
    res = shard.gather(local, mine, world)
    if rank == 0:
        q.put(res)
    dist.destroy_process_group()


def test_two_rank_gather_equals_single_rank():
    from minim_gb300 import abi
    from oracle.oracle import Oracle
    from tests.workloads import lj_cluster
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert len(res) == len(SIZES)
    for i, (e, it, x) in enumerate(res):
        o = Oracle(abi.lj(), lj_cluster(SIZES[i], seed=i))
        r = o.minimise(abi.minimiser("lbfgs", tol=1e-6))
        assert e == r.energy and it == r.iter and np.array_equal(np.array(x), o.coords)
