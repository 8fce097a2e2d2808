"""The allocation-free LJ minimisation entry point
(minim_gpu_lj_minimise_noalloc): same results as the batch kernel with 256
threads per CTA, on two calls in a row through the one fixed scratch array,
and no device memory taken by the calls themselves.

This file is named to be collected last, so it also runs after every other
GPU test in the same process."""
import numpy as np
import pytest

from minim_gb300 import abi, runtime
from tests.workloads import lj_cluster

pytestmark = pytest.mark.gpu


def _batch_reference(p, x0, mp):
    inst = runtime.Instance(p, x0)
    b = runtime.Batch()
    b.add(inst, mp)
    r = b.run(threads=256)[0]
    return r, inst.coords


def _device(torch, x0):
    return torch.tensor(np.asarray(x0, dtype=np.float64).ravel(), device="cuda")


def _noalloc(torch, p, x, mp):
    stream = torch.cuda.current_stream().cuda_stream
    r = runtime.lj_minimise_noalloc(p, x.data_ptr(), x.numel(), mp, stream)
    return r


def test_noalloc_matches_batch_two_calls():
    torch = pytest.importorskip("torch")
    p = abi.lj()
    # a large L-BFGS cluster, then a smaller FIRE one: the second call runs on
    # scratch left dirty by the first
    cases = [
        (lj_cluster(150, seed=901), abi.minimiser("lbfgs", m=8, tol=1e-6)),
        (lj_cluster(38, seed=902), abi.minimiser("fire", linesearch="backtracking", dt_max=0.0,
                                                 tol=1e-6, max_iter=200000)),
    ]
    refs = [_batch_reference(p, x0, mp) for x0, mp in cases]
    xs = [_device(torch, x0) for x0, _ in cases]
    warm = _device(torch, cases[1][0])
    # the first call on the device looks up the scratch array's address
    _noalloc(torch, p, warm, cases[1][1])
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    res = [_noalloc(torch, p, x, mp) for x, (_, mp) in zip(xs, cases)]
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    outs = [(r, x.cpu().numpy()) for r, x in zip(res, xs)]
    for (rr, xr), (rn, xn) in zip(refs, outs):
        assert rr.status == abi.RES_CONVERGED
        assert rn.status == rr.status
        assert rn.iter == rr.iter and rn.evals == rr.evals and rn.fp64_iters == rr.fp64_iters
        assert rn.energy == rr.energy
        assert np.array_equal(xn, xr)
    # the two calls took no device memory (the tensors were made before free0)
    assert free1 == free0


def test_noalloc_rejects_oversize():
    torch = pytest.importorskip("torch")
    p = abi.lj()
    x0 = lj_cluster(1025, seed=903)
    with pytest.raises(runtime.MinimGpuError) as e:
        _noalloc(torch, p, _device(torch, x0), abi.minimiser("lbfgs", tol=1e-6))
    assert e.value.code == abi.ERR_INVALID
    assert "3072" in str(e.value)
