"""Seeded synthetic inputs shared by the tests, the smoke check and bench.py.

Random numbers come from numpy's MT19937 bit generator (seeded through
numpy's SeedSequence); raw 64-bit draws are mapped to [0,1) as
(r >> 11) * 2^-53, so the sequences are fully specified and identical on
every platform.
"""
import numpy as np


class Rng:
    """Uniform [0,1) doubles from raw 64-bit MT19937 draws."""

    def __init__(self, seed):
        self.g = np.random.Generator(np.random.MT19937(seed))

    def uniform(self, n=None):
        k = 1 if n is None else n
        r = self.g.integers(0, 2 ** 64, size=k, dtype=np.uint64, endpoint=False)
        u = (r >> np.uint64(11)).astype(np.float64) * 2.0 ** -53
        return u[0] if n is None else u

    def normal(self, n):
        u1 = np.maximum(self.uniform(n), 2.0 ** -53)
        u2 = self.uniform(n)
        return np.sqrt(-2 * np.log(u1)) * np.cos(2 * np.pi * u2)


def lj_cluster(n, seed=0, density=0.5, rmin=0.8, ndim=3):
    """Particles uniform in a cube of side (n/density)^(1/3), rejecting any
    draw closer than rmin to an earlier particle."""
    rng = Rng(seed)
    side = (n / density) ** (1.0 / ndim)
    pts = np.zeros((n, ndim))
    k = 0
    while k < n:
        p = rng.uniform(ndim) * side
        if k == 0 or np.min(np.sum((pts[:k] - p) ** 2, axis=1)) >= rmin * rmin:
            pts[k] = p
            k += 1
    return pts.ravel()


def pf_noise(grid, seed=0, amp=0.05, nfluid=1):
    rng = Rng(seed)
    n = int(np.prod(grid)) * nfluid
    return (rng.uniform(n) * 2 - 1) * amp


def pf_simplex(grid, nfluid=3, seed=0):
    """Per-node random point on the simplex (sorted-uniform spacings)."""
    rng = Rng(seed)
    ng = int(np.prod(grid))
    u = np.sort(rng.uniform(ng * (nfluid - 1)).reshape(ng, nfluid - 1), axis=1)
    edges = np.concatenate([np.zeros((ng, 1)), u, np.ones((ng, 1))], axis=1)
    return np.diff(edges, axis=1).ravel()


def sheet(k, seed=0, jitter=0.05, amp=0.1):
    """k x k regular triangulated square sheet: (flat jittered coordinates,
    triangles, coordinates with a Gaussian out-of-plane perturbation)."""
    rng = Rng(seed)
    ij = np.array([(i, j) for i in range(k) for j in range(k)], dtype=np.float64)
    xy = ij + (rng.uniform(2 * k * k).reshape(-1, 2) * 2 - 1) * jitter
    flat = np.concatenate([xy, np.zeros((k * k, 1))], axis=1).ravel()
    tris = []
    for i in range(k - 1):
        for j in range(k - 1):
            a = i * k + j
            b, c = a + 1, a + k
            d = c + 1
            tris += [[a, c, b], [b, c, d]]
    pert = flat.copy()
    pert[2::3] += rng.normal(k * k) * amp
    return flat, np.array(tris, dtype=np.int32), pert


# --- pf-pillar-collapse (reference test/benchmark/pf-pillar-collapse/main.cpp) ---
# A ternary field on an 80 x 100 x 1 grid: fluid 0 is a diffused solid (a base
# of height 9.5 and two pillars reaching y < 79, spacing 40 between them), fluid
# 1 a liquid above y = 79, fluid 2 gas.  A pressure on the liquid pushes it into
# the gap; the critical pressure at which it reaches the base is found by
# bisection and compared with -2 gamma cos(theta) / (spacing * resolution).
PILLAR = dict(nx=80, ny=100, res=1e-3, y_top=20, y_bottom=9.5, gamma=100.0)


def pillar_solid(spacing=40.0):
    """The sharp solid mask (main.cpp initialiseSolid)."""
    nx, ny = PILLAR["nx"], PILLAR["ny"]
    x, y = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    width = nx - spacing
    base = y < PILLAR["y_bottom"]
    pillar = (y < ny - 1 - PILLAR["y_top"]) & ((x <= width / 2) | (x > nx - 1 - width / 2))
    return (base | pillar).astype(np.uint8).ravel()


def pillar_kwargs(contact_angle, pressure=None, diffuse=False):
    """PhaseField keyword arguments (minim_gb300.abi.phase_field) of the run at
    one contact angle: diffuse=True gives diffuseSolid's potential (confinement
    100 on fluid 0, no density constraint); otherwise fluid 0 is fixed, the
    density constraint hard and the liquid under ``pressure``."""
    nx, ny, g = PILLAR["nx"], PILLAR["ny"], PILLAR["gamma"]
    dg = g * np.cos(np.deg2rad(contact_angle))
    walls = np.zeros((nx, ny), np.uint8)
    walls[:, 0] = walls[:, ny - 1] = 1
    kw = dict(grid=[nx, ny, 1], nfluid=3, resolution=PILLAR["res"],
              surface_tension=[g - dg / 2, g + dg / 2, g], solid=walls.ravel())
    if diffuse:
        kw.update(confinement=[100.0, 0.0, 0.0], density_constraint="none")
    else:
        kw.update(pressure=[0.0, float(pressure), 0.0], fix_fluid=[1, 0, 0],
                  density_constraint="hard")
    return kw


def pillar_diffuse_init(solid):
    x = np.zeros(3 * solid.size)
    x[0::3] = solid
    return x


def pillar_fluid(diffused):
    """The initial field from the diffused solid (main.cpp initialiseFluid)."""
    nx, ny = PILLAR["nx"], PILLAR["ny"]
    s = np.asarray(diffused).reshape(-1, 3)[:, 0]
    y = np.tile(np.arange(ny), nx)
    liquid = (y > ny - 1 - PILLAR["y_top"]).astype(float)
    x = np.zeros((s.size, 3))
    x[:, 0] = s
    x[:, 1] = liquid * (1 - s)
    x[:, 2] = (1 - liquid) * (1 - s)
    return x.ravel()


def pillar_failed(coords):
    """Liquid has reached 5 nodes above the base at the centre (main.cpp checkFailed)."""
    y = int(PILLAR["y_bottom"] + 5)
    k = ((PILLAR["nx"] - 1) // 2) * PILLAR["ny"] + y
    return bool(np.asarray(coords)[3 * k + 1] > 0.5)


def pillar_analytic(contact_angle, spacing=40.0):
    return -2 * PILLAR["gamma"] * np.cos(np.deg2rad(contact_angle)) / (spacing * PILLAR["res"])


PILLAR_ANGLES = (30, 50, 70, 90, 110, 130, 150)


def pillar_bisect(run, n):
    """The critical-pressure bisection of main.cpp run(), for n contact angles
    in lockstep: ``run(idx, p)`` minimises angle idx[k] at pressure p[k] and
    returns (failed, iterations) per run.  The bounds start at +-0.1 gamma /
    res; a failed run lowers the upper bound, a held one raises the lower;
    an angle is done when the half-width is at most 1e-3 of the start."""
    pmax = 0.1 * PILLAR["gamma"] / PILLAR["res"]
    lo, hi = np.full(n, -pmax), np.full(n, pmax)
    hist = [[] for _ in range(n)]
    for _ in range(50):
        idx = [i for i in range(n) if abs(hi[i] - lo[i]) / 2 > 1e-3 * pmax]
        if not idx:
            break
        p = 0.5 * (lo[idx] + hi[idx])
        for i, pi, (failed, it) in zip(idx, p, run(idx, p)):
            hist[i].append((float(pi), bool(failed), int(it)))
            if failed:
                hi[i] = pi
            else:
                lo[i] = pi
    return lo, hi, hist
