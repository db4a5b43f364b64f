"""Every compile-time z plan of the complex FP32 fused z pass (-m gpu).

For each padded z length a box can produce (Pz = smallest 5-smooth >= 2 nz,
nz = 1..256) the FP32 block MVP, which runs the compile-time plan, must agree
with the FP64 block MVP (runtime plan, itself checked against the oracle) to
the FP32 tolerance, and a few boxes are checked against the oracle directly.
"""
import numpy as np
import pytest

import bdda
from oracle import mbt

pytestmark = pytest.mark.gpu

TOL32 = 5e-6


def _smooth_at_least(v):
    while True:
        t = v
        for p in (2, 3, 5):
            while t % p == 0:
                t //= p
        if t == 1:
            return v
        v += 1


def _nz_per_pz():
    seen = {}
    for nz in range(1, 257):
        seen.setdefault(_smooth_at_least(2 * nz), nz)
    return sorted(seen.items())


def _mvp(op, x, L, n3, prec, dt):
    import torch
    xd = torch.from_numpy(np.ascontiguousarray(x.T)).to(dt).cuda()
    yd = torch.zeros_like(xd)
    torch.cuda.synchronize()
    op.mvp_device(xd.data_ptr(), yd.data_ptr(), L, n3, n3, prec=prec)
    torch.cuda.synchronize()
    return yd.cpu().numpy().T.astype(np.complex128)


def test_every_z_plan_fp32_vs_fp64():
    import torch
    rng = np.random.default_rng(5)
    worst = (0.0, None)
    for i, (Pz, nz) in enumerate(_nz_per_pz()):
        n = (3, 2, nz)
        N = int(np.prod(n))
        nocc = max(1, (2 * N) // 3)
        addr = np.sort(rng.choice(N, size=nocc, replace=False)).astype(np.int32)
        L = 1 + i % 3  # odd counts leave the last right-hand-side pair of the packed z pass half empty
        x = rng.standard_normal((3 * nocc, L)) + 1j * rng.standard_normal((3 * nocc, L))
        op = bdda.Operator(n, 0.03, 2 * np.pi / 0.55)
        op.set_dipoles(addr)
        assert op.info()[0][2] == Pz
        y64 = _mvp(op, x, L, 3 * nocc, bdda.PREC_FP64, torch.complex128)
        y32 = _mvp(op, x, L, 3 * nocc, bdda.PREC_FP32, torch.complex64)
        if nocc == 1:
            assert np.max(np.abs(y32)) == 0.0
            continue
        rel = np.linalg.norm(y32 - y64) / np.linalg.norm(y64)
        if rel > worst[0]:
            worst = (rel, Pz)
        assert rel < TOL32, (Pz, nz, rel)


@pytest.mark.parametrize("L", [3, 8])
def test_every_z_plan_pipelined_and_scalar_kernels(L):
    """The pipelined z pass (bulk copies of rows, spectrum and twiddles into
    shared memory, persistent CTAs) against the scalar kernel on every z
    length, fused and unfused plans: the same arithmetic (agreement to FP32
    rounding), and both against the FP64 MVP.  L = 3 leaves CTA warps of the
    pipelined kernel without a task in the last round of a line; L = 8 fills
    them."""
    import torch
    rng = np.random.default_rng(11 + L)
    for i, (Pz, nz) in enumerate(_nz_per_pz()):
        n = (4, 3, nz)
        N = int(np.prod(n))
        nocc = max(2, (2 * N) // 3)
        addr = np.sort(rng.choice(N, size=nocc, replace=False)).astype(np.int32)
        x = rng.standard_normal((3 * nocc, L)) + 1j * rng.standard_normal((3 * nocc, L))
        op = bdda.Operator(n, 0.03, 2 * np.pi / 0.55)
        op.set_dipoles(addr)
        op.set_autotune(False)
        y64 = _mvp(op, x, L, 3 * nocc, bdda.PREC_FP64, torch.complex128)
        op.set_z_kernel("pipelined")
        yp = _mvp(op, x, L, 3 * nocc, bdda.PREC_FP32, torch.complex64)
        op.set_z_kernel("scalar")
        ys = _mvp(op, x, L, 3 * nocc, bdda.PREC_FP32, torch.complex64)
        op.check_status()
        ref = np.linalg.norm(y64)
        assert np.linalg.norm(yp - y64) / ref < TOL32, (Pz, nz)
        assert np.linalg.norm(yp - ys) / ref < 1e-6, (Pz, nz)


def _to_df(a):  # complex128 -> float32 [..., 4] = (re_hi, re_lo, im_hi, im_lo)
    hi_r = a.real.astype(np.float32)
    hi_i = a.imag.astype(np.float32)
    lo_r = (a.real - hi_r.astype(np.float64)).astype(np.float32)
    lo_i = (a.imag - hi_i.astype(np.float64)).astype(np.float32)
    return np.stack([hi_r, lo_r, hi_i, lo_i], axis=-1)


def test_every_z_plan_double_float_vs_fp64():
    """The double-float z pass (residual MVPs of mixed solves) runs the same
    compile-time plans; it must give FP64-level results on every length."""
    import torch
    rng = np.random.default_rng(9)
    for i, (Pz, nz) in enumerate(_nz_per_pz()):
        n = (2, 3, nz)
        N = int(np.prod(n))
        nocc = max(2, (2 * N) // 3)
        addr = np.sort(rng.choice(N, size=nocc, replace=False)).astype(np.int32)
        L = 1 + i % 2
        x = rng.standard_normal((3 * nocc, L)) + 1j * rng.standard_normal((3 * nocc, L))
        op = bdda.Operator(n, 0.03, 2 * np.pi / 0.55)
        op.set_dipoles(addr)
        y64 = _mvp(op, x, L, 3 * nocc, bdda.PREC_FP64, torch.complex128)
        xd = torch.from_numpy(np.ascontiguousarray(_to_df(x.T))).cuda()
        yd = torch.zeros_like(xd)
        torch.cuda.synchronize()
        op.mvp_device(xd.data_ptr(), yd.data_ptr(), L, 3 * nocc, 3 * nocc, prec=bdda.PREC_DF64)
        torch.cuda.synchronize()
        y = yd.cpu().numpy().astype(np.float64)
        ydf = ((y[..., 0] + y[..., 1]) + 1j * (y[..., 2] + y[..., 3])).T
        rel = np.linalg.norm(ydf - y64) / np.linalg.norm(y64)
        assert rel < 1e-12, (Pz, nz, rel)


@pytest.mark.parametrize("n", [(4, 3, 60), (2, 5, 75), (3, 3, 128), (2, 2, 256)])
def test_z_plan_fp32_vs_oracle(n):
    import torch
    rng = np.random.default_rng(sum(n))
    N = int(np.prod(n))
    nocc = N // 2
    addr = np.sort(rng.choice(N, size=nocc, replace=False)).astype(np.int32)
    L = 3
    x = rng.standard_normal((3 * nocc, L)) + 1j * rng.standard_normal((3 * nocc, L))
    lf, k = 0.021, 2 * np.pi / 0.55
    gh, P = mbt.green_hat(n, 3, lf, k)
    ref = mbt.block_mvp(n, 3, gh, P, addr, np.zeros(3 * nocc, complex), x)
    op = bdda.Operator(n, lf, k)
    op.set_dipoles(addr)
    y32 = _mvp(op, x, L, 3 * nocc, bdda.PREC_FP32, torch.complex64)
    assert np.linalg.norm(y32 - ref) / np.linalg.norm(ref) < TOL32
