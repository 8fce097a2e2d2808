"""ctypes mirror of the C ABI declared in include/minim_gpu.h (types only).

Nothing here loads a library.  ``Params`` helpers turn keyword arguments
named like the reference's setters into the ABI's parameter structs while
keeping the numpy arrays they point at alive.
"""
import ctypes as C

import numpy as np

# call status
OK, ERR_INVALID, ERR_RUNTIME, ERR_CUDA, ERR_OOM, ERR_NO_DEVICE, ERR_BUSY = range(7)
# per-instance result status
RES_CONVERGED, RES_MAXITER, RES_NAN, RES_TIMEOUT, RES_CANCELLED, RES_RUNNING, RES_REJECTED = range(7)
RES_NAMES = {0: "converged", 1: "maxiter", 2: "nan", 3: "timeout", 4: "cancelled",
             5: "running", 6: "rejected"}
# potential kinds (PFU: PhaseFieldUnstructured, the element form of PhaseField)
LJ, PF, BAH, PFU = 0, 1, 2, 3
# PhaseField density constraints
DENSITY = {"hard": 0, "gradient": 0, "soft": 1, "energy penalty": 1, "none": 2, "fixed": 3}
# minimisers, line searches, precision
LBFGS, FIRE, GD, ANNEAL = 0, 1, 2, 3
LS_BACKTRACKING, LS_NONE = 0, 1
PREC_MIXED, PREC_FP64, PREC_FP32 = 0, 1, 2
# minim_gpu_eval_kernel paths: the kernels of a minimiser stage
EVAL_FP32_GRID, EVAL_FP32_CTA, EVAL_FP64S_GRID, EVAL_FP64S_CTA, EVAL_LINES, EVAL_LINES_TMA = range(6)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_cp = C.c_char_p


class LjParams(C.Structure):
    _fields_ = [("ndim", C.c_int), ("sigma", C.c_double), ("epsilon", C.c_double), ("cutoff", C.c_double)]


class PfParams(C.Structure):
    _fields_ = [
        ("grid", C.c_int * 3), ("nfluid", C.c_int), ("resolution", C.c_double),
        ("n_interface_size", C.c_int), ("interface_size", _dp),
        ("n_surface_tension", C.c_int), ("surface_tension", _dp),
        ("density_constraint", C.c_int), ("density_const", C.c_double),
        ("volume_fixed", C.c_int), ("vol_const", C.c_double), ("volume", _dp),
        ("pressure", _dp), ("solid", C.c_void_p),
        ("n_contact_angle", C.c_int), ("contact_angle", _dp),
        ("force", _dp), ("fix_fluid", C.c_void_p), ("confinement", _dp),
    ]


class BahParams(C.Structure):
    _fields_ = [
        ("ntri", C.c_int), ("tris", _ip),
        ("nbond", C.c_int), ("bonds", _ip), ("bond_stride", C.c_int),
        ("nhinge", C.c_int), ("hinges", _ip), ("hinge_stride", C.c_int),
        ("modulus", C.c_double), ("poisson_ratio", C.c_double),
        ("n_thickness", C.c_int), ("thickness", _dp),
        ("n_kbond", C.c_int), ("kbond", _dp),
        ("n_khinge", C.c_int), ("khinge", _dp),
        ("n_length0", C.c_int), ("length0", _dp),
        ("n_theta0", C.c_int), ("theta0", _dp),
        ("n_force", C.c_int), ("force", _dp),
        ("wall_on", C.c_int), ("wall_adhesion", C.c_int),
        ("wall_epsilon", C.c_double), ("wall_sigma", C.c_double),
    ]


class MinimiserParams(C.Structure):
    _fields_ = [
        ("method", C.c_int), ("linesearch", C.c_int), ("max_iter", C.c_int),
        ("tol", C.c_double), ("m", C.c_int), ("max_step", C.c_double),
        ("init_step", C.c_double), ("dt_max", C.c_double), ("alpha", C.c_double),
        ("precision", C.c_int),
        ("temp_init", C.c_double), ("displacement", C.c_double), ("cooling_rate", C.c_double),
        ("max_rejections", C.c_int), ("n_temp_schedule", C.c_int), ("temp_schedule", _dp),
        ("seed", C.c_uint64),
    ]


class Result(C.Structure):
    _fields_ = [
        ("status", C.c_int), ("iter", C.c_int), ("fp64_iters", C.c_int), ("evals", C.c_int),
        ("energy", C.c_double), ("rms", C.c_double), ("dt_max", C.c_double),
        ("latency_ms", C.c_double), ("run_ms", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class RunStats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("wall_ms", C.c_double), ("launches", C.c_int64),
                ("abytes", C.c_double), ("pairs32", C.c_double), ("pairs64", C.c_double),
                ("iterations", C.c_int64), ("fp64_iterations", C.c_int64),
                ("switches", C.c_int64 * 4), ("phase_ms", C.c_double * 3), ("tune_ms", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("max_bytes", C.c_size_t), ("max_slots", C.c_int), ("slice_iters", C.c_int),
                ("threads_per_cta", C.c_int)]


def _f64(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())


def _i32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.int32).ravel())


def _u8(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint8).ravel())


class Params:
    """A potential description: ``kind`` plus the ABI struct and the arrays it
    points at.  Build with :func:`lj`, :func:`phase_field` or
    :func:`bar_and_hinge`."""

    def __init__(self, kind, struct, keep):
        self.kind = kind
        self.struct = struct
        self._keep = keep

    def ptr(self):
        return C.cast(C.pointer(self.struct), C.c_void_p)


def lj(ndim=3, sigma=1.0, epsilon=1.0, cutoff=0.0):
    """LjNd(nDim, sigma, epsilon); cutoff > 0 keeps only the pairs closer
    than it (LjNd::setCutoff, no counterpart in the reference)."""
    return Params(LJ, LjParams(ndim, sigma, epsilon, cutoff), [])


def phase_field(grid, nfluid=1, resolution=1.0, interface_size=None, surface_tension=None,
                density_constraint="hard", density_const=1.0, volume_fixed=False,
                vol_const=0.01, volume=None, pressure=None, solid=None, contact_angle=None,
                force=None, fix_fluid=None, confinement=None):
    """PhaseField with the reference's setter names and defaults."""
    s = PfParams()
    keep = []
    s.grid[:] = list(grid)
    s.nfluid = nfluid
    s.resolution = resolution

    def arr(name, value, conv, count_field=None, ptr_type=_dp):
        if value is None:
            if count_field:
                setattr(s, count_field, 0)
            return
        a = conv(value)
        keep.append(a)
        if ptr_type is C.c_void_p:
            setattr(s, name, a.ctypes.data_as(C.c_void_p))
        else:
            setattr(s, name, a.ctypes.data_as(ptr_type))
        if count_field:
            setattr(s, count_field, a.size)

    if interface_size is not None and np.ndim(interface_size) == 0:
        interface_size = [interface_size] * nfluid
    if surface_tension is not None and np.ndim(surface_tension) == 0:
        surface_tension = [surface_tension] * nfluid
    arr("interface_size", interface_size, _f64, "n_interface_size")
    arr("surface_tension", surface_tension, _f64, "n_surface_tension")
    s.density_constraint = DENSITY[density_constraint] if isinstance(density_constraint, str) \
        else int(density_constraint)
    s.density_const = density_const
    s.volume_fixed = int(bool(volume_fixed))
    s.vol_const = vol_const
    arr("volume", volume, _f64)
    arr("pressure", pressure, _f64)
    arr("solid", solid, _u8, ptr_type=C.c_void_p)
    if contact_angle is not None and np.ndim(contact_angle) == 0:
        contact_angle = [contact_angle] * (int(np.prod(grid)) * nfluid)
    arr("contact_angle", contact_angle, _f64, "n_contact_angle")
    if force is not None:
        f = np.asarray(force, dtype=np.float64)
        if f.ndim == 1:
            f = np.tile(f, (nfluid, 1))
        force = f
    arr("force", force, _f64)
    arr("fix_fluid", fix_fluid, _u8, ptr_type=C.c_void_p)
    arr("confinement", confinement, _f64)
    return Params(PF, s, keep)


def phase_field_unstructured(grid, **kw):
    """PhaseFieldUnstructured with the reference's setter names and defaults
    (the same keywords as :func:`phase_field`; ``vol_const`` is the fixed
    volume's penalty strength)."""
    p = phase_field(grid, **kw)
    p.kind = PFU
    return p


def bar_and_hinge(triangulation=None, bonds=None, hinges=None, modulus=1.0, poisson_ratio=0.3,
                  thickness=None, rigidity=None, length0=None, theta0=None, force=None,
                  wall=False, wall_adhesion=False, wall_params=(1e-12, 1e-5)):
    """BarAndHinge with the reference's setter names; ``rigidity`` is
    (kBond, kHinge), each a scalar or an array."""
    s = BahParams()
    keep = []

    def iarr(value, n_field, p_field, stride_field=None):
        if value is None:
            return
        a = np.asarray(value, dtype=np.int32)
        a2 = np.ascontiguousarray(a.reshape(a.shape[0], -1))
        keep.append(a2)
        setattr(s, n_field, a2.shape[0])
        setattr(s, p_field, a2.ctypes.data_as(_ip))
        if stride_field:
            setattr(s, stride_field, a2.shape[1])

    def farr(value, n_field, p_field):
        if value is None:
            return
        a = _f64(np.atleast_1d(value))
        keep.append(a)
        setattr(s, n_field, a.size)
        setattr(s, p_field, a.ctypes.data_as(_dp))

    iarr(triangulation, "ntri", "tris")
    iarr(bonds, "nbond", "bonds", "bond_stride")
    iarr(hinges, "nhinge", "hinges", "hinge_stride")
    s.modulus = modulus
    s.poisson_ratio = poisson_ratio
    farr(thickness, "n_thickness", "thickness")
    if rigidity is not None:
        farr(rigidity[0], "n_kbond", "kbond")
        farr(rigidity[1], "n_khinge", "khinge")
    farr(length0, "n_length0", "length0")
    farr(theta0, "n_theta0", "theta0")
    farr(force, "n_force", "force")
    s.wall_on = int(bool(wall))
    s.wall_adhesion = int(bool(wall_adhesion))
    s.wall_epsilon, s.wall_sigma = wall_params
    return Params(BAH, s, keep)


_METHODS = {"lbfgs": LBFGS, "fire": FIRE, "gd": GD, "graddescent": GD, "anneal": ANNEAL}


def minimiser(method="lbfgs", linesearch=None, max_iter=100000, tol=-1.0, m=5, max_step=0.0,
              init_step=1.0, dt_max=0.0, alpha=0.1, precision="mixed", temp_init=1.0,
              displacement=0.1, cooling_rate=1.0, max_rejections=0, temp_schedule=None, seed=0):
    """Minimiser parameters with the reference defaults.  ``linesearch`` None
    takes the reference default: backtracking, except Fire with an explicit
    dtMax (the ``Fire(dtMax)`` constructor) which uses none.  Anneal takes
    ``temp_init``, ``displacement`` (its constructor's arguments),
    ``cooling_rate``, ``max_rejections``, an optional tabulated
    ``temp_schedule`` and the random ``seed``."""
    meth = _METHODS[method.lower()] if isinstance(method, str) else int(method)
    if linesearch is None:
        ls = LS_NONE if (meth == FIRE and dt_max != 0) else LS_BACKTRACKING
    else:
        ls = {"backtracking": LS_BACKTRACKING, "none": LS_NONE}[linesearch] \
            if isinstance(linesearch, str) else int(linesearch)
    prec = {"mixed": PREC_MIXED, "fp64": PREC_FP64, "fp32": PREC_FP32}[precision] \
        if isinstance(precision, str) else int(precision)
    mp = MinimiserParams(meth, ls, max_iter, tol, m, max_step, init_step, dt_max, alpha, prec,
                         temp_init, displacement, cooling_rate, max_rejections, 0, None, seed)
    if temp_schedule is not None:
        ts = _f64(temp_schedule)
        mp._keep = ts
        mp.n_temp_schedule = ts.size
        mp.temp_schedule = ts.ctypes.data_as(_dp)
    return mp
