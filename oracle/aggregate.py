"""Oracle: the seeded lattice aggregates of the benchmark workloads -- TEST
INFRASTRUCTURE ONLY.

The reference ships its aggregates only as target files (``DDA_target_*.out``);
the tool that grew them is not in its tree.  The benchmark workloads therefore
use the library's own seeded generator (``bdda_aggregate``: tunable
particle-cluster aggregation on the simple cubic lattice, Filippov et al.
2000).  This module restates that generator step for step in plain Python so
that the CPU reference arm of the benchmark can build exactly the same target
without loading the CUDA library.  ``tests/test_oracle.py`` pins it
site-for-site against ``bdda.aggregate``.

Algorithm: monomer N+1 is attached to a face-adjacent empty site of the
cluster; 48 frontier sites are drawn (splitmix64, uniform index), and the one
whose distance from the current centre of mass is nearest to
G = sqrt((N+1)^2/N Rg(N+1)^2 - (N+1) Rg(N)^2), Rg(N) = (N/kf)^(1/Df), wins
(first of equals).  The frontier is a list with swap-with-last removal, so its
order -- and with it the draw -- is deterministic.
"""
from __future__ import annotations

import math

import numpy as np

_MASK = (1 << 64) - 1
_GOLD = 0x9E3779B97F4A7C15
_SAMPLE = 48


class _SplitMix:
    def __init__(self, seed: int):
        self.s = (seed * _GOLD + 0x2545F4914F6CDD1D) & _MASK

    def uniform(self) -> float:
        self.s = (self.s + _GOLD) & _MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        z ^= z >> 31
        return float(z >> 11) * (1.0 / 9007199254740992.0)


def aggregate(nocc: int, kf: float = 1.0, Df: float = 2.8, seed: int = 1):
    """(n, address): box (nx, ny, nz) and 0-based addresses ny nz ix + nz iy + iz
    of the sites in the order they were attached (same as ``bdda.aggregate``)."""
    rng = _SplitMix(int(seed))
    xs, ys, zs = [], [], []
    occ = set()
    frontier = []
    fpos = {}
    nb = ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))
    sums = [0.0, 0.0, 0.0]

    def add_site(x, y, z):
        k = (x, y, z)
        occ.add(k)
        i = fpos.pop(k, None)
        if i is not None:
            last = frontier[-1]
            frontier[i] = last
            if last != k:
                fpos[last] = i
            frontier.pop()
        for dx, dy, dz in nb:
            q = (x + dx, y + dy, z + dz)
            if q in occ or q in fpos:
                continue
            fpos[q] = len(frontier)
            frontier.append(q)
        xs.append(x)
        ys.append(y)
        zs.append(z)
        sums[0] += x
        sums[1] += y
        sums[2] += z

    def rg(N):
        return math.pow(N / kf, 1.0 / Df)

    add_site(0, 0, 0)
    while len(xs) < nocc:
        N = float(len(xs))
        cx, cy, cz = sums[0] / N, sums[1] / N, sums[2] / N
        g2 = (N + 1) * (N + 1) / N * rg(N + 1) * rg(N + 1) - (N + 1) * rg(N) * rg(N)
        g = math.sqrt(max(0.0, g2))
        best = frontier[0]
        bestd = 1e300
        m = len(frontier)
        for _ in range(min(_SAMPLE, m)):
            q = frontier[int(rng.uniform() * m) % m]
            d = math.sqrt((q[0] - cx) * (q[0] - cx) + (q[1] - cy) * (q[1] - cy) + (q[2] - cz) * (q[2] - cz))
            e = abs(d - g)
            if e < bestd:
                bestd = e
                best = q
        add_site(*best)
    x = np.array(xs, dtype=np.int64)
    y = np.array(ys, dtype=np.int64)
    z = np.array(zs, dtype=np.int64)
    n = (int(x.max() - x.min() + 1), int(y.max() - y.min() + 1), int(z.max() - z.min() + 1))
    address = n[1] * n[2] * (x - x.min()) + n[2] * (y - y.min()) + (z - z.min())
    return n, address.astype(np.int32)


def directions(n_dirs: int, seed: int):
    """Seeded propagation directions with two orthonormal polarisations each,
    as the benchmark workloads draw them (``bdda.directions``): the first is +z,
    the others uniform on the sphere (normalised numpy PCG64 normals).
    Returns (uinc, einc) for L = 2 n_dirs."""
    rng = np.random.default_rng(seed)
    us, es = [], []
    for i in range(n_dirs):
        if i == 0:
            u = np.array([0.0, 0.0, 1.0])
        else:
            v = rng.standard_normal(3)
            u = v / np.linalg.norm(v)
        a = np.array([1.0, 0.0, 0.0]) if abs(u[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
        e1 = a - np.dot(a, u) * u
        e1 /= np.linalg.norm(e1)
        e2 = np.cross(u, e1)
        us += [u, u]
        es += [e1.astype(np.complex128), e2.astype(np.complex128)]
    return np.array(us), np.array(es)
