"""ctypes front end of the CPU checkers (test infrastructure only).

* ``Oracle``    -- the plain-C FP64 restatement (oracle/libminim_oracle.so).
* ``Reference`` -- the reference library compiled from its own sources plus
  oracle/ref_shim.cpp (oracle/_ref/libminim_ref.so); present only where the
  reference tree was available at build time.

Both take the same ``minim_gb300.abi.Params`` descriptions as the GPU engine.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from minim_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "libminim_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libminim_ref.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


def build_oracle(quiet=True):
    """Compile the restatement (and nothing else)."""
    out = subprocess.run(["make", "-C", HERE, "oracle"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)


_lib = None
_ref = None


def _load_oracle():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        lib = C.CDLL(ORACLE_SO)
        lib.oracle_last_error.restype = C.c_char_p
        lib.oracle_create.argtypes = [C.c_int, C.c_void_p, _dp, C.c_size_t, _ip, C.c_int,
                                      C.POINTER(C.c_void_p)]
        lib.oracle_destroy.argtypes = [C.c_void_p]
        lib.oracle_default_tol.argtypes = [C.c_void_p]
        lib.oracle_default_tol.restype = C.c_double
        lib.oracle_set_coords.argtypes = [C.c_void_p, _dp]
        lib.oracle_get_coords.argtypes = [C.c_void_p, _dp]
        lib.oracle_energy_gradient.argtypes = [C.c_void_p, _dp, _dp, _dp]
        lib.oracle_apply_constraints.argtypes = [C.c_void_p, _dp]
        lib.oracle_minimise.argtypes = [C.c_void_p, C.POINTER(abi.MinimiserParams),
                                        C.POINTER(abi.Result)]
        lib.oracle_bah_elements.argtypes = [C.c_void_p, _ip, C.POINTER(_ip), C.POINTER(_dp), _ip,
                                            C.POINTER(_ip), C.POINTER(_dp)]
        lib.oracle_pf_internals.argtypes = [C.c_void_p, C.POINTER(_dp), C.POINTER(_dp),
                                            C.POINTER(_dp), C.POINTER(_dp), _ip]
        lib.oracle_set_threads.argtypes = [C.c_void_p, C.c_int]
        lib.oracle_anneal_libc.argtypes = [C.c_void_p, C.POINTER(abi.MinimiserParams), C.c_uint,
                                           C.POINTER(abi.Result)]
        _lib = lib
    return _lib


def reference_available():
    return os.path.exists(REF_SO)


def _load_ref():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise RuntimeError("reference library not built (oracle/_ref/libminim_ref.so)")
        lib = C.CDLL(REF_SO)
        lib.ref_create.argtypes = [C.c_int, C.c_void_p, _dp, C.c_size_t, _ip, C.c_int,
                                   C.POINTER(C.c_void_p)]
        lib.ref_destroy.argtypes = [C.c_void_p]
        lib.ref_last_error.argtypes = [C.c_char_p, C.c_size_t]
        lib.ref_set_num_threads.argtypes = [C.c_int]
        lib.ref_default_tol.argtypes = [C.c_void_p]
        lib.ref_default_tol.restype = C.c_double
        lib.ref_set_coords.argtypes = [C.c_void_p, _dp]
        lib.ref_get_coords.argtypes = [C.c_void_p, _dp]
        lib.ref_energy_gradient.argtypes = [C.c_void_p, _dp, _dp, _dp]
        lib.ref_apply_constraints.argtypes = [C.c_void_p, _dp]
        lib.ref_minimise.argtypes = [C.c_void_p, C.POINTER(abi.MinimiserParams),
                                     C.POINTER(abi.Result)]
        lib.ref_bah_elements.argtypes = [C.c_void_p, C.c_int, _ip, _ip, _dp, _ip, _ip, _dp]
        lib.ref_pf_internals.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp, _ip]
        lib.ref_set_num_threads(1)
        _ref = lib
    return _ref


def _vec(x):
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel())


class _Base:
    def __init__(self, params, x0, fixed=None):
        self.params = params
        self.x0 = _vec(x0)
        self.ndof = self.x0.size
        fx = np.ascontiguousarray(np.asarray(fixed if fixed is not None else [], dtype=np.int32))
        self._fixed = fx
        h = C.c_void_p()
        rc = self._create(params.kind, params.ptr(), self.x0.ctypes.data_as(_dp), self.ndof,
                          fx.ctypes.data_as(_ip), fx.size, C.byref(h))
        if rc != 0:
            raise ValueError(self._error())
        self.h = h

    def energy_gradient(self, x=None, energy=True, gradient=True):
        xv = None if x is None else _vec(x)
        e = C.c_double(0.0)
        g = np.zeros(self.ndof) if gradient else None
        self._eg(self.h, None if xv is None else xv.ctypes.data_as(_dp),
                 C.byref(e) if energy else None, None if g is None else g.ctypes.data_as(_dp))
        return (e.value if energy else None), g

    def energy(self, x=None):
        return self.energy_gradient(x, gradient=False)[0]

    def gradient(self, x=None):
        return self.energy_gradient(x, energy=False)[1]

    def apply_constraints(self, v):
        a = _vec(v).copy()
        self._ac(self.h, a.ctypes.data_as(_dp))
        return a

    @property
    def coords(self):
        x = np.zeros(self.ndof)
        self._get(self.h, x.ctypes.data_as(_dp))
        return x

    @coords.setter
    def coords(self, x):
        xv = _vec(x)
        self._set(self.h, xv.ctypes.data_as(_dp))

    def minimise(self, mp):
        r = abi.Result()
        rc = self._min(self.h, C.byref(mp), C.byref(r))
        if rc != 0:
            raise RuntimeError(self._error())
        return r


class Oracle(_Base):
    """FP64 C restatement of the reference path."""

    def __init__(self, params, x0, fixed=None, threads=1):
        """threads > 1 runs the PhaseField evaluation and the minimisers'
        vector loops on that many host threads (CPU-baseline timing only);
        the default 1 keeps the reference's serial summation order."""
        lib = _load_oracle()
        self._lib = lib
        self._create = lib.oracle_create
        self._eg = lib.oracle_energy_gradient
        self._ac = lib.oracle_apply_constraints
        self._get = lib.oracle_get_coords
        self._set = lib.oracle_set_coords
        self._min = lib.oracle_minimise
        super().__init__(params, x0, fixed)
        if threads > 1:
            lib.oracle_set_threads(self.h, int(threads))

    def _error(self):
        return self._lib.oracle_last_error().decode()

    def anneal_libc(self, mp):
        """Anneal drawing its random numbers from the C library's rand()
        after srand(mp.seed), in the reference's order: the same run as the
        reference library's with the same seed."""
        r = abi.Result()
        rc = self._lib.oracle_anneal_libc(self.h, C.byref(mp), C.c_uint(mp.seed & 0xFFFFFFFF), C.byref(r))
        if rc != 0:
            raise RuntimeError(self._error())
        return r

    @property
    def default_tol(self):
        return self._lib.oracle_default_tol(self.h)

    def bah_elements(self):
        nb, nh = C.c_int(), C.c_int()
        b, h = _ip(), _ip()
        bp, hp = _dp(), _dp()
        self._lib.oracle_bah_elements(self.h, C.byref(nb), C.byref(b), C.byref(bp), C.byref(nh),
                                      C.byref(h), C.byref(hp))
        bars = np.ctypeslib.as_array(b, (max(nb.value, 1) * 2,))[: 2 * nb.value].reshape(-1, 2).copy()
        bpar = np.ctypeslib.as_array(bp, (max(nb.value, 1) * 2,))[: 2 * nb.value].reshape(-1, 2).copy()
        hin = np.ctypeslib.as_array(h, (max(nh.value, 1) * 4,))[: 4 * nh.value].reshape(-1, 4).copy()
        hpar = np.ctypeslib.as_array(hp, (max(nh.value, 1) * 2,))[: 2 * nh.value].reshape(-1, 2).copy()
        return bars, bpar, hin, hpar

    def pf_internals(self):
        k, kp, nv, sa = _dp(), _dp(), _dp(), _dp()
        nk = C.c_int()
        self._lib.oracle_pf_internals(self.h, C.byref(k), C.byref(kp), C.byref(nv), C.byref(sa),
                                      C.byref(nk))
        ng = int(np.prod(self.params.struct.grid[:]))
        a = lambda p, n: np.ctypeslib.as_array(p, (n,)).copy()
        return a(k, nk.value), a(kp, nk.value), a(nv, ng), a(sa, ng)

    def __del__(self):
        try:
            self._lib.oracle_destroy(self.h)
        except Exception:
            pass


class Reference(_Base):
    """The reference library itself (serial build, one OpenMP thread)."""

    def __init__(self, params, x0, fixed=None, threads=1):
        lib = _load_ref()
        lib.ref_set_num_threads(threads)
        self._lib = lib
        self._create = lib.ref_create
        self._eg = lib.ref_energy_gradient
        self._ac = lib.ref_apply_constraints
        self._get = lib.ref_get_coords
        self._set = lib.ref_set_coords
        self._min = lib.ref_minimise
        super().__init__(params, x0, fixed)

    def _error(self):
        buf = C.create_string_buffer(512)
        self._lib.ref_last_error(buf, 512)
        return buf.value.decode()

    @property
    def default_tol(self):
        return self._lib.ref_default_tol(self.h)

    def bah_elements(self):
        cap = 4 * self.ndof + 64
        nb, nh = C.c_int(), C.c_int()
        b = np.zeros(2 * cap, np.int32)
        h = np.zeros(4 * cap, np.int32)
        bp = np.zeros(2 * cap)
        hp = np.zeros(2 * cap)
        self._lib.ref_bah_elements(self.h, cap, C.byref(nb), b.ctypes.data_as(_ip),
                                   bp.ctypes.data_as(_dp), C.byref(nh), h.ctypes.data_as(_ip),
                                   hp.ctypes.data_as(_dp))
        return (b[: 2 * nb.value].reshape(-1, 2), bp[: 2 * nb.value].reshape(-1, 2),
                h[: 4 * nh.value].reshape(-1, 4), hp[: 2 * nh.value].reshape(-1, 2))

    def pf_internals(self):
        ng = int(np.prod(self.params.struct.grid[:]))
        nf = self.params.struct.nfluid
        k = np.zeros(ng * nf + 8)
        kp = np.zeros(ng * nf + 8)
        nv = np.zeros(ng)
        sa = np.zeros(ng)
        nk = C.c_int()
        self._lib.ref_pf_internals(self.h, k.ctypes.data_as(_dp), kp.ctypes.data_as(_dp),
                                   nv.ctypes.data_as(_dp), sa.ctypes.data_as(_dp), C.byref(nk))
        return k[: nk.value], kp[: nk.value], nv, sa

    def __del__(self):
        try:
            self._lib.ref_destroy(self.h)
        except Exception:
            pass
