"""Block MVP on the GPU against the oracle (parity tests, -m gpu).

FP64 path: relative L2 error <= 1e-12 against the oracle's FP64 3-D FFT and
the literal restatement of the reference's 1-D MBT_fft_mvp.
FP32 path: relative L2 error <= 5e-6 (complex FP32 FFT over the padded grid).
"""
import numpy as np
import pytest

import bdda
from oracle import mbt

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 5e-6


def _torch():
    import torch
    return torch


def _dev(a, dtype):
    """host (n x L) complex matrix -> device tensor laid out column-major (L, n)."""
    torch = _torch()
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).to(dtype).cuda()


def _host(t):
    return t.cpu().numpy().T


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("n", [(3, 2, 4), (5, 4, 3), (1, 1, 5), (6, 6, 7), (2, 9, 1), (7, 3, 5)])
def test_mbt_fft_mvp_matches_literal_reference(n):
    rng = np.random.default_rng(sum(n))
    lf, k = 0.37, 2.1 + 0.05j
    N = int(np.prod(n))
    x = rng.standard_normal(3 * N) + 1j * rng.standard_normal(3 * N)
    ref = mbt.mbt_fft_mvp(n, 3, mbt.mbt_fft_init(n, 3, lf, k), x)
    op = bdda.Operator(n, lf, k, prec=bdda.PREC_FP64)
    y = op.mbt_fft_mvp(x)
    assert _rel(y, ref) < TOL64


def _aggregate_case(nocc, seed, L):
    n, addr = bdda.aggregate(nocc, 1.0, 2.8, seed)
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((3 * nocc, L)) + 1j * rng.standard_normal((3 * nocc, L))
    diag = rng.standard_normal(3 * nocc) + 1j * rng.standard_normal(3 * nocc) + 5.0
    return n, addr, x, diag


@pytest.mark.parametrize("nocc,L", [(1, 1), (2, 3), (57, 2), (300, 1), (300, 16), (700, 32)])
@pytest.mark.parametrize("mode", ["offdiag", "diag", "jacobi"])
def test_block_mvp_fp64_and_fp32_vs_oracle(nocc, L, mode):
    torch = _torch()
    n, addr, x, diag = _aggregate_case(nocc, 11 + nocc, L)
    lf, k = 0.021, 2 * np.pi / 0.55
    gh, P = mbt.green_hat(n, 3, lf, k)
    jpre = 1.0 / diag
    ref = mbt.block_mvp(n, 3, gh, P, addr, diag if mode != "offdiag" else np.zeros_like(diag), x,
                        jpre if mode == "jacobi" else None)
    op = bdda.Operator(n, lf, k)
    op.set_dipoles(addr)
    assert op.info()[0] == P
    for prec, dt, tol in ((bdda.PREC_FP64, torch.complex128, TOL64), (bdda.PREC_FP32, torch.complex64, TOL32)):
        xd = _dev(x, dt)
        yd = torch.zeros_like(xd)
        dd = torch.from_numpy(diag).to(dt).cuda()
        jd = torch.from_numpy(jpre).to(dt).cuda()
        torch.cuda.synchronize()
        op.mvp_device(xd.data_ptr(), yd.data_ptr(), L, 3 * nocc, 3 * nocc, prec=prec,
                      diag=dd.data_ptr() if mode != "offdiag" else None,
                      jpre=jd.data_ptr() if mode == "jacobi" else None)
        torch.cuda.synchronize()
        got = _host(yd)
        if nocc == 1 and mode == "offdiag":
            assert np.max(np.abs(got)) == 0.0
        else:
            assert _rel(got, ref) < tol, (prec, _rel(got, ref))


def test_block_mvp_leading_dimension_and_in_place():
    torch = _torch()
    n, addr, x, diag = _aggregate_case(400, 5, 5)
    lf, k = 0.03, 8.0
    gh, P = mbt.green_hat(n, 3, lf, k)
    ref = mbt.block_mvp(n, 3, gh, P, addr, diag, x)
    op = bdda.Operator(n, lf, k, prec=bdda.PREC_FP64)
    op.set_dipoles(addr)
    ld = 3 * 400 + 7
    buf = torch.zeros((5, ld), dtype=torch.complex128, device="cuda")
    buf[:, : 3 * 400] = _dev(x, torch.complex128)
    dd = torch.from_numpy(diag).cuda()
    torch.cuda.synchronize()
    op.mvp_device(buf.data_ptr(), buf.data_ptr(), 5, ld, ld, diag=dd.data_ptr())   # y overwrites x
    torch.cuda.synchronize()
    got = buf[:, : 3 * 400].cpu().numpy().T
    assert _rel(got, ref) < TOL64
    assert torch.all(buf[:, 3 * 400:] == 0)


def test_block_mvp_large_box_linearity_and_precisions():
    """A 16384-dipole aggregate: FP32 vs FP64 agreement, linearity, and one column vs the oracle."""
    torch = _torch()
    nocc, L = 16384, 4
    n, addr, x, diag = _aggregate_case(nocc, 3, L)
    lf, k = 0.0184, 2 * np.pi / 0.55
    op = bdda.Operator(n, lf, k)
    op.set_dipoles(addr)
    x64 = _dev(x, torch.complex128)
    y64 = torch.zeros_like(x64)
    x32 = x64.to(torch.complex64)
    y32 = torch.zeros_like(x32)
    torch.cuda.synchronize()
    op.mvp_device(x64.data_ptr(), y64.data_ptr(), L, 3 * nocc, 3 * nocc, prec=bdda.PREC_FP64)
    op.mvp_device(x32.data_ptr(), y32.data_ptr(), L, 3 * nocc, 3 * nocc, prec=bdda.PREC_FP32)
    torch.cuda.synchronize()
    a64, a32 = _host(y64), _host(y32)
    assert _rel(a32, a64) < TOL32
    # linearity: A(2 x0 - 3i x1) = 2 A x0 - 3i A x1 (columns 0 and 1)
    comb = _dev((2 * x[:, 0] - 3j * x[:, 1])[:, None], torch.complex128)
    yc = torch.zeros_like(comb)
    torch.cuda.synchronize()
    op.mvp_device(comb.data_ptr(), yc.data_ptr(), 1, 3 * nocc, 3 * nocc, prec=bdda.PREC_FP64)
    torch.cuda.synchronize()
    assert _rel(_host(yc)[:, 0], 2 * a64[:, 0] - 3j * a64[:, 1]) < TOL64
    gh, P = mbt.green_hat(n, 3, lf, k)
    ref0 = mbt.mvp3d(n, 3, gh, P, x[:, 0], addr)
    assert _rel(a64[:, 0], ref0) < TOL64


def test_block_mvp_rejects_bad_arguments():
    op = bdda.Operator((4, 4, 4), 0.1, 3.0, prec=bdda.PREC_FP32)
    with pytest.raises(bdda.BddaError):
        op.set_dipoles([0, 5, 5])                    # duplicate site
    with pytest.raises(bdda.BddaError):
        op.set_dipoles([0, 64])                      # outside the box
    op.set_dipoles([0, 1, 2])
    torch = _torch()
    x = torch.zeros((1, 9), dtype=torch.complex128, device="cuda")
    with pytest.raises(bdda.BddaError):                  # FP64 tables absent
        op.mvp_device(x.data_ptr(), x.data_ptr(), 1, 9, 9, prec=bdda.PREC_FP64)


def test_block_mvp_double_float_vs_oracle():
    """Double-float (FP32 hi/lo pairs) MVP used for mixed-precision residuals: FP64-level accuracy."""
    torch = _torch()
    nocc, L = 900, 6
    n, addr, x, diag = _aggregate_case(nocc, 31, L)
    lf, k = 0.021, 2 * np.pi / 0.55
    gh, P = mbt.green_hat(n, 3, lf, k)
    ref = mbt.block_mvp(n, 3, gh, P, addr, diag, x)
    op = bdda.Operator(n, lf, k)
    op.set_dipoles(addr)

    def to_df(a):   # complex128 (rows, cols) -> float32 [..., 4] = (re_hi, re_lo, im_hi, im_lo)
        hi_r = a.real.astype(np.float32)
        hi_i = a.imag.astype(np.float32)
        lo_r = (a.real - hi_r.astype(np.float64)).astype(np.float32)
        lo_i = (a.imag - hi_i.astype(np.float64)).astype(np.float32)
        return np.stack([hi_r, lo_r, hi_i, lo_i], axis=-1)

    xd = torch.from_numpy(np.ascontiguousarray(to_df(x.T))).cuda()
    dd = torch.from_numpy(np.ascontiguousarray(to_df(diag))).cuda()
    yd = torch.zeros_like(xd)
    torch.cuda.synchronize()
    op.mvp_device(xd.data_ptr(), yd.data_ptr(), L, 3 * nocc, 3 * nocc, prec=bdda.PREC_DF64, diag=dd.data_ptr())
    torch.cuda.synchronize()
    y = yd.cpu().numpy().astype(np.float64)
    got = ((y[..., 0] + y[..., 1]) + 1j * (y[..., 2] + y[..., 3])).T
    assert _rel(got, ref) < TOL64
