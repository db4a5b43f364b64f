"""Oracle: the f=3 Green-tensor operator as a complex128 3-D FFT in PyTorch --
TEST INFRASTRUCTURE ONLY.

A second oracle for sizes the numpy restatement cannot reach in seconds (the
N=65536 aggregates): the same 2x-padded circulant embedding as
``oracle.mbt.green_grid`` (the Green block of ``mvp_fft/application_function.cpp:21-40``
on offsets j < n, j - P for j > P - n, zero gap and zero at d = 0), transformed
with ``torch.fft`` in complex128 on whichever device the tensors live (the GPU
in the large parity tests).  It shares no code with the CUDA library: the
kernels under test are checked against it, and it is itself checked against
``oracle.mbt.mvp3d`` on small boxes (``tests/test_oracle.py``).
"""
from __future__ import annotations

import numpy as np


def _offsets(torch, ni, pi, device):
    o = torch.zeros(pi, dtype=torch.float64, device=device)
    valid = torch.zeros(pi, dtype=torch.bool, device=device)
    o[:ni] = torch.arange(ni, dtype=torch.float64, device=device)
    valid[:ni] = True
    if ni > 1:
        o[pi - ni + 1:] = torch.arange(pi - ni + 1, pi, dtype=torch.float64, device=device) - pi
        valid[pi - ni + 1:] = True
    return o, valid


class GreenOperator:
    """y = A_off x for the occupied sites ``address`` of box n (f = 3)."""

    def __init__(self, n, lf, k, address, device="cpu", P=None):
        import torch
        from oracle import mbt
        self.torch = torch
        self.n = tuple(int(v) for v in n)
        self.P = tuple(P) if P is not None else mbt.padded_grid(self.n)
        self.device = torch.device(device)
        k = complex(k)
        comps = []
        valids = []
        for i in range(3):
            o, v = _offsets(torch, self.n[i], self.P[i], self.device)
            shape = [1, 1, 1]
            shape[i] = self.P[i]
            comps.append((o * lf).reshape(shape))
            valids.append(v.reshape(shape))
        dx, dy, dz = comps
        valid = valids[0] & valids[1] & valids[2]
        r2 = dx * dx + dy * dy + dz * dz
        mask = valid & (r2 > 0)
        r = torch.sqrt(torch.where(mask, r2, torch.ones_like(r2)))
        kk = torch.tensor(k, dtype=torch.complex128, device=self.device)
        e = torch.exp(1j * kk * r) / r
        c1 = kk * kk
        c2 = (1.0 - 1j * kk * r) / r / r
        d = (dx, dy, dz)
        self.ghat = torch.zeros((3, 3) + self.P, dtype=torch.complex128, device=self.device)
        for a in range(3):
            for b in range(a, 3):
                rr = (d[a] * d[b]) / (r * r)
                delta = 1.0 if a == b else 0.0
                g = -(c1 * (delta - rr) - c2 * (delta - 3.0 * rr)) * e
                g = torch.where(mask, g, torch.zeros((), dtype=torch.complex128, device=self.device))
                gh = torch.fft.fftn(g.expand(self.P).contiguous(), dim=(0, 1, 2))
                self.ghat[a, b] = gh
                if b != a:
                    self.ghat[b, a] = gh
            del rr
        address = np.asarray(address, dtype=np.int64)
        ny, nz = self.n[1], self.n[2]
        ix = address // (ny * nz)
        iy = (address // nz) % ny
        iz = address % nz
        self.idx = tuple(torch.from_numpy(v).to(self.device) for v in (ix, iy, iz))
        self.nocc = address.size

    def apply(self, x):
        """A_off x for x of shape (3 nocc, L) (numpy or torch, complex128); returns a torch tensor."""
        torch = self.torch
        x = torch.as_tensor(x, dtype=torch.complex128).to(self.device)
        if x.dim() == 1:
            x = x[:, None]
        ix, iy, iz = self.idx
        out = torch.empty_like(x)
        for l in range(x.shape[1]):
            grid = torch.zeros((3,) + self.P, dtype=torch.complex128, device=self.device)
            xv = x[:, l].reshape(-1, 3)
            for c in range(3):
                grid[c, ix, iy, iz] = xv[:, c]
            xh = torch.fft.fftn(grid, dim=(1, 2, 3))
            del grid
            yh = torch.einsum("abxyz,bxyz->axyz", self.ghat, xh)
            del xh
            yg = torch.fft.ifftn(yh, dim=(1, 2, 3))
            del yh
            out[:, l] = torch.stack([yg[c, ix, iy, iz] for c in range(3)], dim=1).reshape(-1)
        return out

    def true_residual(self, diag, B, X):
        """Per-column ||b - (diag o x + A_off x)|| / ||b|| (numpy float64 array)."""
        torch = self.torch
        Bt = torch.as_tensor(np.asarray(B), dtype=torch.complex128).to(self.device)
        Xt = torch.as_tensor(np.asarray(X), dtype=torch.complex128).to(self.device)
        dt = torch.as_tensor(np.asarray(diag), dtype=torch.complex128).to(self.device)
        R = Bt - (dt[:, None] * Xt + self.apply(Xt))
        num = torch.linalg.vector_norm(R, dim=0)
        den = torch.linalg.vector_norm(Bt, dim=0)
        return (num / den).cpu().numpy()


def relative_error(a, b):
    """||a - b|| / ||b|| of two arrays (numpy or torch)."""
    a = np.asarray(a.cpu() if hasattr(a, "cpu") else a)
    b = np.asarray(b.cpu() if hasattr(b, "cpu") else b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))

