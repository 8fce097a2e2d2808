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
