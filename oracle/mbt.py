"""Oracle: the multilevel block-Toeplitz (MBT) Green-tensor operator on the CPU.

Test infrastructure only (see ``oracle/__init__.py``).  Three independent
formulations of ``y = A_off x`` on a cuboid lattice ``n = (nx, ny, nz)`` with the
reference's site ordering ``address = ny*nz*ix + nz*iy + iz``
(``Target_manager.cpp:98``) and dipole-major component interleaving (row
``f*site + c``):

1. ``mbt_fft_init`` / ``mbt_fft_mvp`` -- a literal restatement of the
   reference's 1-D MBT projection (``mvp_fft/BT_fft.cpp``, ``BT_pad.cpp``,
   ``BT_reconstruct.cpp``, ``MBT_fft_init.cpp``, ``MBT_fft_mvp.cpp``), with
   numpy's FFT standing in for FFTW (same sign convention: forward e^{-i},
   backward unnormalised, the reference divides by the length).
2. ``dense_matrix`` -- O(N^2) assembly of ``A(r_k - r_m)``, ``k != m``.
3. ``mvp3d`` -- the 2x-padded 3-D circulant embedding that the GPU path uses.

All arithmetic is complex128.
"""
from __future__ import annotations

import numpy as np


def application_function(d, f: int, lf: float, k: complex) -> np.ndarray:
    """f x f block A(r) for a lattice offset ``d`` (3 ints), r = d*lf.

    Restates ``mvp_fft/application_function.cpp:21-70``:
    f=3: ``-G`` with G = e^{ikr}/r [k^2 (I - r^ r^) - (1 - ikr)/r^2 (I - 3 r^ r^)]
    (``:36-39``); f=6: ``[[-G, -F], [F, -G]]`` with
    F = -k^2 e^{ikr}/r (1 - 1/(ikr)) [r^]x (``:63-67``).  r = 0 gives a zero
    block (``:31-34``, ``:46-49``).
    """
    x = np.asarray(d, dtype=np.float64) * lf
    r = float(np.sqrt(np.dot(x, x)))
    if f not in (3, 6):
        raise ValueError("unknown f value")
    if r == 0.0:
        return np.zeros((f, f), dtype=np.complex128)
    xx = np.outer(x, x)
    eye = np.eye(3)
    g = k * k * (eye - xx / r / r)
    g = g - ((1.0 - 1j * k * r) / r / r) * (eye - 3.0 * xx / r / r)
    g = g * np.exp(1j * k * r) / r
    if f == 3:
        return -g
    u = x / r
    ux = np.array([[0.0, -u[2], u[1]], [u[2], 0.0, -u[0]], [-u[1], u[0], 0.0]])
    fm = -k * k * (np.exp(1j * k * r) / r) * (1.0 - 1.0 / (1j * k * r)) * ux
    out = np.zeros((6, 6), dtype=np.complex128)
    out[:3, :3] = -g
    out[:3, 3:] = -fm
    out[3:, :3] = fm
    out[3:, 3:] = -g
    return out


# --------------------------------------------------------------------------
# 1. literal 1-D MBT projection
# --------------------------------------------------------------------------

def bt_fft(n, f, n_ind, level, lf, k, leaf=None):
    """Recursive MBT projection vector ``Au`` (``mvp_fft/BT_fft.cpp:8-53``).

    ``n_ind`` is a 2 x M integer array of 1-based block positions; at each level
    the lower+diagonal children (row index this_n..1, column 1) come first
    (``:39-44``), then the upper children (row 1, column 2..this_n) (``:46-50``).
    The leaf is ``flipud`` + transpose of the f x f block flattened in Eigen's
    column-major order (``:25-31``), i.e. ``leaf[r*f + c] = A[f-1-r, c]``.
    ``leaf`` optionally replaces ``application_function`` (used by the f=1
    known-answer test of ``mvp_fft_example.cpp:37-103``).
    """
    n = list(n)
    m = len(n)
    if level == m + 1:
        if leaf is not None:
            a = np.atleast_2d(np.asarray(leaf(n_ind), dtype=np.complex128))
        else:
            d = n_ind[0, :] - n_ind[1, :]
            a = application_function(d, f, lf, k)
        a = a[::-1, :]            # flipud
        a = a.T                   # transpose
        return a.flatten(order="F")
    len_au = f * f * int(np.prod([2 * v - 1 for v in n[level - 1:]]))
    au = np.zeros(len_au, dtype=np.complex128)
    this_n = n[level - 1]
    b_edge = f * f * int(np.prod([2 * v - 1 for v in n[level:]]))
    n_ind = n_ind.copy()
    for i in range(this_n, 0, -1):
        n_ind[1, level - 1] = 1
        n_ind[0, level - 1] = i
        blk = bt_fft(n, f, n_ind, level + 1, lf, k, leaf)
        au[b_edge * (this_n - i): b_edge * (this_n - i) + b_edge] = blk
    for i in range(2, this_n + 1):
        n_ind[1, level - 1] = i
        blk = bt_fft(n, f, n_ind, level + 1, lf, k, leaf)
        au[b_edge * (i + this_n - 2): b_edge * (i + this_n - 2) + b_edge] = blk
    return au


def bt_pad(n, f, x):
    """Scatter a cuboid vector into the MBT-projected layout (``mvp_fft/BT_pad.cpp:6-45``)."""
    n = list(n)
    x = np.asarray(x)
    if len(n) < 1:
        return np.concatenate([x, np.zeros(f * f - f, dtype=x.dtype)])
    b_edge = f * int(np.prod(n[1:]))
    parts = []
    for i in range(1, n[0] + 1):
        blk = bt_pad(n[1:], f, x[(i - 1) * b_edge: i * b_edge])
        parts.append(blk)
        if len(n) > 1:
            nz = (n[1] - 1) * f * f * int(np.prod([2 * v - 1 for v in n[2:]]))
            parts.append(np.zeros(nz, dtype=x.dtype))
    return np.concatenate(parts)


def bt_reconstruct(n, f, bz):
    """Gather the cuboid result from the MBT layout (``mvp_fft/BT_reconstruct.cpp:5-36``)."""
    n = list(n)
    if len(n) < 1:
        return np.array([bz[i - 1] for i in range(f, f * f + 1, f)], dtype=bz.dtype)
    b_edge = f * f * int(np.prod([2 * v - 1 for v in n[1:]]))
    parts = []
    for i in range(n[0], 2 * n[0]):
        parts.append(bt_reconstruct(n[1:], f, bz[(i - 1) * b_edge: i * b_edge]))
    return np.concatenate(parts)


def mbt_fft_init(n, f, lf, k, leaf=None):
    """``Au_til = FFT(reverse(BT_fft(...)))`` (``mvp_fft/MBT_fft_init.cpp:22-35``)."""
    n = list(n)
    fft_length = f * f * int(np.prod([2 * v - 1 for v in n]))
    n_ind = np.ones((2, len(n)), dtype=np.int64)
    au = bt_fft(n, f, n_ind, 1, lf, k, leaf)
    if au.size != fft_length:
        raise RuntimeError("wrong Au size !")
    return np.fft.fft(au[::-1])


def mbt_fft_mvp(n, f, au_til, p_hat):
    """One off-diagonal matvec on the cuboid vector (``mvp_fft/MBT_fft_mvp.cpp:19-32``)."""
    fft_length = au_til.size
    z = bt_pad(n, f, np.asarray(p_hat, dtype=np.complex128))
    pz = np.zeros(fft_length, dtype=np.complex128)
    pz[: z.size] = z
    q = np.fft.ifft(au_til * np.fft.fft(pz))   # ifft already divides by the length
    return bt_reconstruct(n, f, q)


# --------------------------------------------------------------------------
# 2. dense assembly
# --------------------------------------------------------------------------

def site_coords(n):
    """Lattice coordinates (ix, iy, iz) of every cuboid site in address order."""
    nx, ny, nz = n
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    return np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1)


def dense_matrix(n, f, lf, k, address=None):
    """Dense ``A_off`` over the sites ``address`` (all cuboid sites by default)."""
    coords = site_coords(n)
    if address is not None:
        coords = coords[np.asarray(address)]
    ns = coords.shape[0]
    a = np.zeros((f * ns, f * ns), dtype=np.complex128)
    cache = {}
    for i in range(ns):
        for j in range(ns):
            d = tuple(int(v) for v in coords[i] - coords[j])
            blk = cache.get(d)
            if blk is None:
                blk = application_function(d, f, lf, k)
                cache[d] = blk
            a[f * i: f * i + f, f * j: f * j + f] = blk
    return a


# --------------------------------------------------------------------------
# 3. 2x-padded 3-D FFT formulation (what the GPU computes)
# --------------------------------------------------------------------------

def smooth235(v: int) -> int:
    """Smallest 2^a 3^b 5^c >= v."""
    while True:
        t = v
        for p in (2, 3, 5):
            while t % p == 0:
                t //= p
        if t == 1:
            return v
        v += 1


def padded_grid(n):
    """Padded grid P_i = smallest 5-smooth >= 2 n_i."""
    return tuple(smooth235(2 * int(v)) for v in n)


def green_grid(n, P, f, lf, k):
    """Circulant embedding of A(d) on the padded grid, shape (f, f, Px, Py, Pz).

    Index j_i maps to the offset j_i (j_i < n_i), j_i - P_i (j_i > P_i - n_i),
    and to a zero block otherwise.
    """
    def offsets(ni, pi):
        o = np.full(pi, np.iinfo(np.int64).min, dtype=np.int64)
        o[:ni] = np.arange(ni)
        o[pi - ni + 1:] = np.arange(pi - ni + 1, pi) - pi
        return o

    ox, oy, oz = (offsets(n[i], P[i]) for i in range(3))
    g = np.zeros((f, f) + tuple(P), dtype=np.complex128)
    dx, dy, dz = np.meshgrid(ox, oy, oz, indexing="ij")
    valid = (dx != np.iinfo(np.int64).min) & (dy != np.iinfo(np.int64).min) & (dz != np.iinfo(np.int64).min)
    dx = np.where(valid, dx, 0).astype(np.float64) * lf
    dy = np.where(valid, dy, 0).astype(np.float64) * lf
    dz = np.where(valid, dz, 0).astype(np.float64) * lf
    r2 = dx * dx + dy * dy + dz * dz
    nz_mask = valid & (r2 > 0)
    r = np.sqrt(np.where(nz_mask, r2, 1.0))
    comps = (dx, dy, dz)
    e = np.exp(1j * k * r) / r
    c1 = k * k
    c2 = (1.0 - 1j * k * r) / r / r
    for a in range(3):
        for b in range(3):
            rr = comps[a] * comps[b] / (r * r)
            delta = 1.0 if a == b else 0.0
            gab = (c1 * (delta - rr) - c2 * (delta - 3.0 * rr)) * e
            g[a, b] = np.where(nz_mask, -gab, 0.0)
    if f == 6:
        u = [c / r for c in comps]
        fac = -k * k * e * (1.0 - 1.0 / (1j * k * r))
        ux = [[0, -u[2], u[1]], [u[2], 0, -u[0]], [-u[1], u[0], 0]]
        for a in range(3):
            for b in range(3):
                fab = np.where(nz_mask, fac * ux[a][b], 0.0) if not isinstance(ux[a][b], int) else 0.0
                g[a, 3 + b] = -fab
                g[3 + a, b] = fab
                g[3 + a, 3 + b] = g[a, b]
    return g


def green_hat(n, f, lf, k, P=None):
    """Forward 3-D FFT of the embedded Green tensor, shape (f, f, Px, Py, Pz)."""
    P = padded_grid(n) if P is None else tuple(P)
    g = green_grid(n, P, f, lf, k)
    return np.fft.fftn(g, axes=(2, 3, 4)), P


def mvp3d(n, f, ghat, P, x, address=None):
    """``y = A_off x`` via the padded 3-D FFT.

    ``x`` is (f*nsites, L) or (f*nsites,) in dipole-major order over ``address``
    (all cuboid sites when None).  Returns the same shape.
    """
    x = np.asarray(x, dtype=np.complex128)
    squeeze = x.ndim == 1
    if squeeze:
        x = x[:, None]
    nx, ny, nz = n
    L = x.shape[1]
    if address is None:
        address = np.arange(nx * ny * nz)
    address = np.asarray(address)
    ix = address // (ny * nz)
    iy = (address // nz) % ny
    iz = address % nz
    y = np.zeros_like(x)
    for l in range(L):
        grid = np.zeros((f,) + tuple(P), dtype=np.complex128)
        xv = x[:, l].reshape(-1, f)
        for c in range(f):
            grid[c, ix, iy, iz] = xv[:, c]
        xh = np.fft.fftn(grid, axes=(1, 2, 3))
        yh = np.einsum("abxyz,bxyz->axyz", ghat, xh)
        yg = np.fft.ifftn(yh, axes=(1, 2, 3))
        yv = np.stack([yg[c, ix, iy, iz] for c in range(f)], axis=1)
        y[:, l] = yv.reshape(-1)
    return y[:, 0] if squeeze else y


def block_mvp(n, f, ghat, P, address, diag, S, jpre=None):
    """Block MVP with the diagonal: ``AS = (DIAG o S + gather(MVP(scatter(S)))) [o jpre]``.

    Restates the inline wrapper of ``bl_krylov_mvp_fft/bl_cocg_rq_jacobi_mvp_fft.cpp:43-60``
    (and ``bl_cocg_rq_mvp_fft.cpp:38-52`` without ``jpre``).
    """
    S = np.asarray(S, dtype=np.complex128)
    out = diag[:, None] * S + mvp3d(n, f, ghat, P, S, address)
    if jpre is not None:
        out = out * jpre[:, None]
    return out
