"""Vectorised CPU restatement of the reference's 1-D MBT FFT matvec, for timing.

Test infrastructure / CPU baseline only.  Same algorithm as ``oracle.mbt``'s
literal recursion (``mvp_fft/BT_fft.cpp``, ``BT_pad.cpp``,
``BT_reconstruct.cpp``, ``MBT_fft_init.cpp``, ``MBT_fft_mvp.cpp``), with the
recursions unrolled into closed-form index maps for three levels:

  BT_pad:        (ix, iy, iz, c) -> ix (2ny-1)(2nz-1) f^2 + iy (2nz-1) f^2 + iz f^2 + c
  BT_reconstruct:(ix, iy, iz, r) <- (nx-1+ix)(2ny-1)(2nz-1) f^2 + (ny-1+iy)(2nz-1) f^2
                                    + (nz-1+iz) f^2 + f r + f - 1
  BT_fft leaf s = (s1, s2, s3) holds A(d) with d_i = n_i - 1 - s_i, flattened
  row-major after flipud: leaf[r f + c] = A[f-1-r, c].

``MbtCpu.block_mvp`` applies it to L right-hand sides in parallel over RHS
(the reference's ``#pragma omp parallel for`` over columns,
``bl_krylov_mvp_fft/bl_cocg_rq_jacobi_mvp_fft.cpp:46-60``) with scipy's FFT
(pocketfft) standing in for FFTW.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import scipy.fft as sfft


def pad_map(n, f):
    nx, ny, nz = n
    ix, iy, iz, c = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), np.arange(f), indexing="ij")
    s2, s3 = 2 * nz - 1, f * f
    return (ix * (2 * ny - 1) * s2 * s3 + iy * s2 * s3 + iz * s3 + c).reshape(-1)


def reconstruct_map(n, f):
    nx, ny, nz = n
    ix, iy, iz, r = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), np.arange(f), indexing="ij")
    s2, s3 = 2 * nz - 1, f * f
    return ((nx - 1 + ix) * (2 * ny - 1) * s2 * s3 + (ny - 1 + iy) * s2 * s3 + (nz - 1 + iz) * s3
            + f * r + f - 1).reshape(-1)


def au_vector(n, lf, k):
    """BT_fft output for f=3, vectorised (``mvp_fft/BT_fft.cpp:8-53``)."""
    nx, ny, nz = n
    f = 3
    s1, s2, s3 = np.meshgrid(np.arange(2 * nx - 1), np.arange(2 * ny - 1), np.arange(2 * nz - 1), indexing="ij")
    d = [(nx - 1 - s1) * lf, (ny - 1 - s2) * lf, (nz - 1 - s3) * lf]
    r2 = d[0] ** 2 + d[1] ** 2 + d[2] ** 2
    zero = r2 == 0
    r = np.sqrt(np.where(zero, 1.0, r2))
    e = np.exp(1j * k * r) / r
    c1 = k * k
    c2 = (1.0 - 1j * k * r) / r / r
    out = np.zeros(s1.shape + (f, f), dtype=np.complex128)
    for a in range(3):
        for b in range(3):
            rr = d[a] * d[b] / (r * r)
            delta = 1.0 if a == b else 0.0
            g = (c1 * (delta - rr) - c2 * (delta - 3.0 * rr)) * e
            out[..., a, b] = np.where(zero, 0.0, -g)
    leaf = out[..., ::-1, :]                    # flipud; leaf[r, c] = A[f-1-r, c]
    return leaf.reshape(-1)


class MbtCpu:
    """The reference's per-RHS FFT matvec on the CPU (FFT length f^2 prod(2n_i-1))."""

    def __init__(self, n, lf, k, address, diag, threads=None):
        self.n = tuple(int(v) for v in n)
        self.f = 3
        au = au_vector(self.n, lf, k)
        self.M = au.size
        self.au_til = sfft.fft(au[::-1])
        self.pmap = pad_map(self.n, 3)
        self.rmap = reconstruct_map(self.n, 3)
        address = np.asarray(address)
        rows = (3 * address[:, None] + np.arange(3)[None, :]).reshape(-1)
        self.rows = rows                   # cuboid rows of the dipole-major compact vector
        self.diag = np.asarray(diag)
        self.threads = threads or os.cpu_count() or 1

    def mvp_cuboid(self, p_hat):
        z = np.zeros(self.M, dtype=np.complex128)
        z[self.pmap] = p_hat
        z = sfft.fft(z, workers=1, overwrite_x=True)
        z *= self.au_til
        z = sfft.ifft(z, workers=1, overwrite_x=True)
        return z[self.rmap]

    def bytes_per_column(self):
        """Host memory one column of ``block_mvp`` holds at its peak, with a
        margin: the padded vector and pocketfft's working copy (16-byte complex;
        measured about 1.9 M x 16 bytes per column at M = 1.39e8)."""
        return int(2.5 * self.M * 16) + 2 * int(np.prod(self.n)) * 3 * 16

    def block_mvp(self, S, cols=None):
        """AS = DIAG o S + gather(MBT_fft_mvp(scatter(S))) over the columns
        ``cols`` (all by default), threaded over columns; other columns of
        the result are left unset."""
        ncub = int(np.prod(self.n)) * 3
        out = np.empty_like(S)

        def col(l):
            p = np.zeros(ncub, dtype=np.complex128)
            p[self.rows] = S[:, l]
            out[:, l] = self.diag * S[:, l] + self.mvp_cuboid(p)[self.rows]

        cols = range(S.shape[1]) if cols is None else cols
        with ThreadPoolExecutor(max_workers=self.threads) as ex:
            list(ex.map(col, cols))
        return out
