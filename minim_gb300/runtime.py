"""ctypes binding of libminim_gb300.so (the C ABI of include/minim_gpu.h).

This is the call path tests and bench.py use: every compute call goes through
the C ABI into the CUDA kernels.  There is no CPU fallback: without the
library or without an sm_103 GPU every call raises.
"""
import ctypes as C
import os

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libminim_gb300.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lib = None

# every symbol declared in include/minim_gpu.h
EXPORTS = [
    "minim_gpu_abi_version", "minim_gpu_last_error", "minim_gpu_default_minimiser",
    "minim_gpu_default_pf", "minim_gpu_default_bah", "minim_gpu_launch_count",
    "minim_gpu_last_run_stats",
    "minim_gpu_instance_create", "minim_gpu_instance_destroy", "minim_gpu_instance_ndof",
    "minim_gpu_instance_default_tol", "minim_gpu_instance_set_coords",
    "minim_gpu_instance_get_coords", "minim_gpu_instance_set_fixed", "minim_gpu_energy_gradient",
    "minim_gpu_apply_constraints", "minim_gpu_minimise", "minim_gpu_batch_create",
    "minim_gpu_batch_add", "minim_gpu_batch_run", "minim_gpu_batch_destroy",
    "minim_gpu_server_create", "minim_gpu_server_submit", "minim_gpu_server_step",
    "minim_gpu_server_poll", "minim_gpu_server_take", "minim_gpu_server_cancel",
    "minim_gpu_server_destroy", "minim_gpu_bah_elements", "minim_gpu_bah_colouring",
    "minim_gpu_pf_setup", "minim_gpu_lj_minimise_noalloc", "minim_gpu_instance_bah_arrays",
    "minim_gpu_eval_kernel", "minim_gpu_tune_table", "minim_gpu_batch_run_shape", "minim_gpu_wait_probe", "minim_gpu_lj_cutoff_pairs",
]


class MinimGpuError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"minim_gpu error {code}: {msg}")
        self.code = code


def load(path=LIB_PATH):
    """Load the engine library (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    lib = C.CDLL(path)
    P = C.c_void_p
    sig = {
        "minim_gpu_abi_version": ([], C.c_int),
        "minim_gpu_last_error": ([C.c_char_p, C.c_size_t], C.c_int),
        "minim_gpu_launch_count": ([], C.c_int64),
        "minim_gpu_last_run_stats": ([C.POINTER(abi.RunStats)], C.c_int),
        "minim_gpu_instance_create": ([C.c_int, P, _dp, C.c_size_t, C.POINTER(P)], C.c_int),
        "minim_gpu_instance_destroy": ([P], C.c_int),
        "minim_gpu_instance_default_tol": ([P, _dp], C.c_int),
        "minim_gpu_instance_set_coords": ([P, _dp], C.c_int),
        "minim_gpu_instance_get_coords": ([P, _dp], C.c_int),
        "minim_gpu_instance_set_fixed": ([P, _ip, C.c_size_t], C.c_int),
        "minim_gpu_energy_gradient": ([P, _dp, _dp, _dp], C.c_int),
        "minim_gpu_apply_constraints": ([P, _dp], C.c_int),
        "minim_gpu_minimise": ([P, C.POINTER(abi.MinimiserParams), C.POINTER(abi.Result)], C.c_int),
        "minim_gpu_batch_create": ([C.POINTER(P)], C.c_int),
        "minim_gpu_batch_add": ([P, P, C.POINTER(abi.MinimiserParams)], C.c_int),
        "minim_gpu_batch_run": ([P, C.c_int, C.POINTER(abi.Result)], C.c_int),
        "minim_gpu_batch_run_shape": ([P, C.c_int, C.c_int, C.POINTER(abi.Result)], C.c_int),
        "minim_gpu_batch_destroy": ([P], C.c_int),
        "minim_gpu_server_create": ([C.POINTER(abi.ServerConfig), C.POINTER(P)], C.c_int),
        "minim_gpu_server_submit": ([P, C.c_int, P, _dp, C.c_size_t, C.POINTER(abi.MinimiserParams),
                                     C.POINTER(C.c_uint64)], C.c_int),
        "minim_gpu_server_step": ([P, _ip, _ip], C.c_int),
        "minim_gpu_server_poll": ([P, C.POINTER(C.c_uint64), C.POINTER(abi.Result), C.c_int, _ip],
                                  C.c_int),
        "minim_gpu_server_take": ([P, C.c_uint64, _dp, C.c_size_t], C.c_int),
        "minim_gpu_server_cancel": ([P, C.c_uint64], C.c_int),
        "minim_gpu_server_destroy": ([P], C.c_int),
        "minim_gpu_bah_elements": ([P, _dp, C.c_size_t, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp],
                                   C.c_int),
        "minim_gpu_bah_colouring": ([P, _dp, C.c_size_t, _ip, _ip, _ip], C.c_int),
        "minim_gpu_pf_setup": ([C.c_int, P, _dp, C.c_size_t, _dp, _dp, _ip, _dp, _dp, _ip], C.c_int),
        "minim_gpu_instance_bah_arrays": ([P, C.c_int, _ip, _ip, _dp, _ip, _ip, _ip, _ip, _dp, _ip, _ip, _ip],
                                          C.c_int),
        "minim_gpu_tune_table": ([C.c_int, _ip, _dp, _ip], C.c_int),
        "minim_gpu_wait_probe": ([C.c_int, _ip, _dp], C.c_int),
        "minim_gpu_lj_cutoff_pairs": ([P, _dp, C.c_int, _ip, _ip], C.c_int),
        "minim_gpu_eval_kernel": ([P, C.c_int, _dp, _dp, C.c_double, _dp, _dp, _dp], C.c_int),
        "minim_gpu_lj_minimise_noalloc": ([P, C.c_void_p, C.c_size_t, C.POINTER(abi.MinimiserParams),
                                           C.POINTER(abi.Result), C.c_void_p], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def _check(rc):
    if rc != 0:
        buf = C.create_string_buffer(1024)
        _lib.minim_gpu_last_error(buf, 1024)
        raise MinimGpuError(rc, buf.value.decode())


def _vec(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel())


def launch_count():
    return load().minim_gpu_launch_count()


def last_run_stats():
    s = abi.RunStats()
    _check(load().minim_gpu_last_run_stats(C.byref(s)))
    d = {k: getattr(s, k) for k, _ in s._fields_}
    d["switches"] = list(s.switches)
    d["phase_ms"] = list(s.phase_ms)
    return d


def wait_probe(limit_ms):
    """Runs the device barrier's bounded wait on a count nothing reaches
    with the given limit: (timed_out, elapsed device ms)."""
    lib = load()
    t, ms = C.c_int(), C.c_double()
    _check(lib.minim_gpu_wait_probe(int(limit_ms), C.byref(t), C.byref(ms)))
    return bool(t.value), ms.value


def tune_table():
    """The autotuner's choices so far: one dict per (kind, size bucket,
    method, precision) key with the chosen threads per CTA and CTAs per
    instance and the measured slice time of each candidate (ms)."""
    lib = load()
    n = C.c_int()
    _check(lib.minim_gpu_tune_table(0, None, None, C.byref(n)))
    k = n.value
    rows = np.zeros(8 * max(k, 1), np.int32)
    ms = np.zeros(8 * max(k, 1))
    _check(lib.minim_gpu_tune_table(k, rows.ctypes.data_as(_ip), ms.ctypes.data_as(_dp), C.byref(n)))
    kinds = {abi.LJ: "lj", abi.PF: "pf", abi.BAH: "bah"}
    out = []
    for i in range(k):
        r = rows[8 * i:8 * i + 8]
        out.append({"kind": kinds.get(int(r[0]), int(r[0])), "bucket": int(r[1]), "method": int(r[2]),
                    "precision": int(r[3]), "threads": int(r[4]), "ctas": int(r[5]), "measured": bool(r[6]),
                    "candidate_ms": [float(v) for v in ms[8 * i:8 * i + int(r[7])]]})
    return out


class Instance:
    """A device-resident State: potential + coordinates (C ABI instance)."""

    def __init__(self, params, x0, fixed=None):
        lib = load()
        self.params = params
        x = _vec(x0)
        self.ndof = x.size
        h = C.c_void_p()
        _check(lib.minim_gpu_instance_create(params.kind, params.ptr(), x.ctypes.data_as(_dp),
                                             x.size, C.byref(h)))
        self.h = h
        if fixed is not None and len(fixed):
            self.set_fixed(fixed)

    def close(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.minim_gpu_instance_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def default_tol(self):
        t = C.c_double()
        _check(_lib.minim_gpu_instance_default_tol(self.h, C.byref(t)))
        return t.value

    @property
    def coords(self):
        return self.get_coords()

    def get_coords(self, out=None):
        """The coordinates into `out` (a contiguous float64 array of ndof, e.g.
        a view of pinned host memory) or a new array."""
        x = np.zeros(self.ndof) if out is None else out
        if x.dtype != np.float64 or not x.flags.c_contiguous or x.size != self.ndof:
            raise ValueError("out must be a contiguous float64 array of ndof values")
        _check(_lib.minim_gpu_instance_get_coords(self.h, x.ctypes.data_as(_dp)))
        return x

    @coords.setter
    def coords(self, x):
        xv = _vec(x)
        _check(_lib.minim_gpu_instance_set_coords(self.h, xv.ctypes.data_as(_dp)))

    def set_fixed(self, idof):
        a = np.ascontiguousarray(np.asarray(idof, dtype=np.int32))
        _check(_lib.minim_gpu_instance_set_fixed(self.h, a.ctypes.data_as(_ip), a.size))

    def energy_gradient(self, x=None, energy=True, gradient=True):
        xv = None if x is None else _vec(x)
        e = C.c_double()
        g = np.zeros(self.ndof) if gradient else None
        _check(_lib.minim_gpu_energy_gradient(
            self.h, None if xv is None else xv.ctypes.data_as(_dp), C.byref(e) if energy else None,
            None if g is None else g.ctypes.data_as(_dp)))
        return (e.value if energy else None), g

    def energy(self, x=None):
        return self.energy_gradient(x, gradient=False)[0]

    def gradient(self, x=None):
        return self.energy_gradient(x, energy=False)[1]

    def eval_kernel(self, path, x, p=None, t=0.0, gradient=True, points=False):
        """One evaluation by a minimiser stage's own kernels at x + t p
        (minim_gpu_eval_kernel; path is one of abi.EVAL_*).  Returns (e, g)
        -- for the line stencils (abi.EVAL_LINES, abi.EVAL_LINES_TMA) each
        holds the two trials (t, t/2) -- and, with
        points (line stencil only), the two points the stencil formed."""
        xv = _vec(x)
        pv = None if p is None else _vec(p)
        two = path in (abi.EVAL_LINES, abi.EVAL_LINES_TMA)
        e = np.zeros(2 if two else 1)
        g = np.zeros((2 if two else 1) * self.ndof) if gradient else None
        xt = np.zeros(2 * self.ndof) if points else None
        _check(_lib.minim_gpu_eval_kernel(self.h, path, xv.ctypes.data_as(_dp),
                                          None if pv is None else pv.ctypes.data_as(_dp), float(t),
                                          e.ctypes.data_as(_dp), None if g is None else g.ctypes.data_as(_dp),
                                          None if xt is None else xt.ctypes.data_as(_dp)))
        if two:
            out = (e, None if g is None else g.reshape(2, self.ndof))
        else:
            out = (e[0], g)
        return out + ((xt.reshape(2, self.ndof),) if points else ())

    def cutoff_pairs(self, x):
        """The pairs (i < j, sorted) that the FP32 stage of this Lennard-Jones
        instance with a cutoff evaluates at x (rounded to FP32)."""
        xv = _vec(x)
        n = C.c_int()
        _check(_lib.minim_gpu_lj_cutoff_pairs(self.h, xv.ctypes.data_as(_dp), 0, None, C.byref(n)))
        cap = max(n.value, 1)
        out = np.zeros(2 * cap, np.int32)
        _check(_lib.minim_gpu_lj_cutoff_pairs(self.h, xv.ctypes.data_as(_dp), cap, out.ctypes.data_as(_ip),
                                              C.byref(n)))
        return out[:2 * n.value].reshape(-1, 2)

    def apply_constraints(self, v):
        a = _vec(v).copy()
        _check(_lib.minim_gpu_apply_constraints(self.h, a.ctypes.data_as(_dp)))
        return a

    def bah_arrays(self):
        """The BarAndHinge elements this instance evaluates, in colour order:
        bars (k, 2), bar_par (k, 2) = {k, l0}, hinges (k, 4), hinge_par (k, 2)
        = {k, theta0}, the colour offsets and whether the device built them."""
        lib = load()
        cnt = [C.c_int() for _ in range(5)]
        _check(lib.minim_gpu_instance_bah_arrays(self.h, 0, C.byref(cnt[0]), None, None, C.byref(cnt[1]), None,
                                                 C.byref(cnt[2]), None, None, C.byref(cnt[3]), None,
                                                 C.byref(cnt[4])))
        nb, nh = cnt[0].value, cnt[2].value
        cap = max(nb, nh, 1)
        bars, bp = np.zeros(2 * cap, np.int32), np.zeros(2 * cap)
        hinges, hp = np.zeros(4 * cap, np.int32), np.zeros(2 * cap)
        boff, hoff = np.zeros(65, np.int32), np.zeros(65, np.int32)
        ncb, nch, dev = C.c_int(), C.c_int(), C.c_int()
        _check(lib.minim_gpu_instance_bah_arrays(
            self.h, cap, C.byref(cnt[0]), bars.ctypes.data_as(_ip), bp.ctypes.data_as(_dp), C.byref(ncb),
            boff.ctypes.data_as(_ip), C.byref(cnt[2]), hinges.ctypes.data_as(_ip), hp.ctypes.data_as(_dp),
            C.byref(nch), hoff.ctypes.data_as(_ip), C.byref(dev)))
        return {"bars": bars[:2 * nb].reshape(-1, 2), "bar_par": bp[:2 * nb].reshape(-1, 2),
                "hinges": hinges[:4 * nh].reshape(-1, 4), "hinge_par": hp[:2 * nh].reshape(-1, 2),
                "bar_off": boff[:ncb.value + 1].copy(), "hinge_off": hoff[:nch.value + 1].copy(),
                "on_device": bool(dev.value)}

    def minimise(self, mp):
        r = abi.Result()
        _check(_lib.minim_gpu_minimise(self.h, C.byref(mp), C.byref(r)))
        return r


class Batch:
    """Many instances minimised together by the persistent batch kernels."""

    def __init__(self):
        lib = load()
        h = C.c_void_p()
        _check(lib.minim_gpu_batch_create(C.byref(h)))
        self.h = h
        self.items = []

    def add(self, inst, mp):
        _check(_lib.minim_gpu_batch_add(self.h, inst.h, C.byref(mp)))
        self.items.append((inst, mp))

    def run(self, threads=0, ctas=0):
        """Runs the batch: autotuned shapes, or `threads` per CTA (and, with
        ctas > 0, that many CTAs per instance) for every instance."""
        res = (abi.Result * len(self.items))()
        if ctas > 0:
            _check(_lib.minim_gpu_batch_run_shape(self.h, threads, ctas, res))
        else:
            _check(_lib.minim_gpu_batch_run(self.h, threads, res))
        return list(res)

    def close(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.minim_gpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous batching: submit requests, step, poll results."""

    def __init__(self, max_bytes=0, max_slots=0, slice_iters=0, threads=0):
        lib = load()
        cfg = abi.ServerConfig(max_bytes, max_slots, slice_iters, threads)
        h = C.c_void_p()
        _check(lib.minim_gpu_server_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.ndof = {}

    def submit(self, params, x0, mp):
        x = _vec(x0)
        rid = C.c_uint64()
        _check(_lib.minim_gpu_server_submit(self.h, params.kind, params.ptr(), x.ctypes.data_as(_dp),
                                            x.size, C.byref(mp), C.byref(rid)))
        self.ndof[rid.value] = x.size
        return rid.value

    def step(self):
        nr, nq = C.c_int(), C.c_int()
        _check(_lib.minim_gpu_server_step(self.h, C.byref(nr), C.byref(nq)))
        return nr.value, nq.value

    def poll(self, max_n=4096):
        ids = (C.c_uint64 * max_n)()
        res = (abi.Result * max_n)()
        n = C.c_int()
        _check(_lib.minim_gpu_server_poll(self.h, ids, res, max_n, C.byref(n)))
        return [(ids[i], res[i]) for i in range(n.value)]

    def take(self, rid):
        x = np.zeros(self.ndof[rid])
        _check(_lib.minim_gpu_server_take(self.h, rid, x.ctypes.data_as(_dp), x.size))
        del self.ndof[rid]
        return x

    def cancel(self, rid):
        _check(_lib.minim_gpu_server_cancel(self.h, rid))

    def close(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.minim_gpu_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- host-only set-up introspection (no GPU needed) ------------------------------
def bah_elements(params, x0):
    lib = load()
    x = _vec(x0)
    cap = 4 * x.size + 64
    nb, nh = C.c_int(), C.c_int()
    b = np.zeros(2 * cap, np.int32)
    h = np.zeros(4 * cap, np.int32)
    bp = np.zeros(2 * cap)
    hp = np.zeros(2 * cap)
    _check(lib.minim_gpu_bah_elements(params.ptr(), x.ctypes.data_as(_dp), x.size, cap, C.byref(nb),
                                      b.ctypes.data_as(_ip), bp.ctypes.data_as(_dp), C.byref(nh),
                                      h.ctypes.data_as(_ip), hp.ctypes.data_as(_dp)))
    return (b[: 2 * nb.value].reshape(-1, 2), bp[: 2 * nb.value].reshape(-1, 2),
            h[: 4 * nh.value].reshape(-1, 4), hp[: 2 * nh.value].reshape(-1, 2))


def bah_colouring(params, x0):
    lib = load()
    x = _vec(x0)
    nb, nh, ok = C.c_int(), C.c_int(), C.c_int()
    _check(lib.minim_gpu_bah_colouring(params.ptr(), x.ctypes.data_as(_dp), x.size, C.byref(nb),
                                       C.byref(nh), C.byref(ok)))
    return nb.value, nh.value, bool(ok.value)


def pf_setup(params, x0):
    lib = load()
    x = _vec(x0)
    s = params.struct
    ng = int(np.prod(s.grid[:]))
    k = np.zeros(ng * s.nfluid + 8)
    kp = np.zeros(ng * s.nfluid + 8)
    nv = np.zeros(ng)
    sa = np.zeros(ng)
    nk, var = C.c_int(), C.c_int()
    _check(lib.minim_gpu_pf_setup(params.kind, params.ptr(), x.ctypes.data_as(_dp), x.size, k.ctypes.data_as(_dp),
                                  kp.ctypes.data_as(_dp), C.byref(nk), nv.ctypes.data_as(_dp),
                                  sa.ctypes.data_as(_dp), C.byref(var)))
    return {"kappa": k[: nk.value], "kappaP": kp[: nk.value], "node_vol": nv, "surface_area": sa,
            "kernel_variant": var.value}


def lj_minimise_noalloc(params, x_dev_ptr, ndof, mp, stream=0):
    """Allocation-free LJ minimisation of the device coordinates at x_dev_ptr
    (ndof doubles, overwritten with the minimum) on `stream` (a cudaStream_t
    handle as an integer, 0 = default stream).  Returns the Result."""
    lib = load()
    r = abi.Result()
    _check(lib.minim_gpu_lj_minimise_noalloc(params.ptr(), C.c_void_p(x_dev_ptr), ndof, C.byref(mp),
                                             C.byref(r), C.c_void_p(stream)))
    return r
