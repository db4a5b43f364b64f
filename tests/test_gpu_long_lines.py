"""Box sides past 256 (padded FFT lines of 513..1200 points) on the GPU (-m gpu).

Lengths past 512 have no compile-time plan: every precision runs the
runtime-plan kernels, whose strided passes drop to one tile buffer where two
of 16-byte elements would not fit in a CTA's shared memory.  Checked against
the oracle's 3-D FFT restatement: the block MVP along each long axis in FP64,
FP32 and double-float, f = 3 and f = 6; a mixed-precision solve on a long rod
reaches its true residual; the request server accepts such boxes.
"""
import numpy as np
import pytest

import bdda
from oracle import krylov, mbt

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _to_df(a):
    hi_r = a.real.astype(np.float32)
    hi_i = a.imag.astype(np.float32)
    lo_r = (a.real - hi_r.astype(np.float64)).astype(np.float32)
    lo_i = (a.imag - hi_i.astype(np.float64)).astype(np.float32)
    return np.stack([hi_r, lo_r, hi_i, lo_i], axis=-1)


def _mvp(op, x, L, n, prec, diag):
    import torch
    if prec == bdda.PREC_DF64:
        xd = torch.from_numpy(np.ascontiguousarray(_to_df(x.T))).cuda()
        dd = torch.from_numpy(np.ascontiguousarray(_to_df(diag))).cuda()
    else:
        dt = torch.complex128 if prec == bdda.PREC_FP64 else torch.complex64
        xd = torch.from_numpy(np.ascontiguousarray(x.T)).to(dt).cuda()
        dd = torch.from_numpy(diag).to(dt).cuda()
    yd = torch.zeros_like(xd)
    torch.cuda.synchronize()
    op.mvp_device(xd.data_ptr(), yd.data_ptr(), L, n, n, prec=prec, diag=dd.data_ptr())
    torch.cuda.synchronize()
    y = yd.cpu().numpy()
    if prec == bdda.PREC_DF64:
        y = y.astype(np.float64)
        return ((y[..., 0] + y[..., 1]) + 1j * (y[..., 2] + y[..., 3])).T
    return y.T.astype(np.complex128)


@pytest.mark.parametrize("n,f", [((300, 3, 4), 3), ((3, 300, 4), 3), ((4, 3, 300), 3), ((520, 2, 3), 3),
                                 ((2, 3, 540), 3), ((290, 2, 2), 6)])
def test_long_axis_mvp_vs_oracle(n, f):
    rng = np.random.default_rng(sum(n) + f)
    N = int(np.prod(n))
    nocc = (3 * N) // 5
    addr = np.sort(rng.choice(N, size=nocc, replace=False)).astype(np.int32)
    L = 3
    rows = f * nocc
    x = rng.standard_normal((rows, L)) + 1j * rng.standard_normal((rows, L))
    diag = rng.standard_normal(rows) + 1j * rng.standard_normal(rows) + 5.0
    lf, k = 0.02, 2 * np.pi / 0.55
    gh, P = mbt.green_hat(n, f, lf, k)
    ref = mbt.block_mvp(n, f, gh, P, addr, diag, x)
    op = bdda.Operator(n, lf, k, f=f)
    op.set_dipoles(addr)
    assert max(op.info()[0]) > 512
    y64 = _mvp(op, x, L, rows, bdda.PREC_FP64, diag)
    assert _rel(y64, ref) < 1e-12
    y32 = _mvp(op, x, L, rows, bdda.PREC_FP32, diag)
    assert _rel(y32, ref) < 5e-6
    ydf = _mvp(op, x, L, rows, bdda.PREC_DF64, diag)
    assert _rel(ydf, ref) < 1e-12


def test_mixed_solve_on_long_rod():
    rng = np.random.default_rng(77)
    n = (420, 5, 5)
    N = int(np.prod(n))
    addr = np.sort(rng.choice(N, size=N // 2, replace=False)).astype(np.int32)
    wl0, m = 0.55, 1.6 + 0.2j
    k = 2 * np.pi / wl0
    lf = 0.5 / (abs(m) * k)
    alpha0 = bdda.polarizability(wl0, lf * (3 / (4 * np.pi)) ** (1 / 3), m * m, k)
    diag = np.full(3 * addr.size, 1.0 / alpha0)
    u, e = bdda.directions(2, 5)
    B = bdda.incident_fields(n, lf, addr, k, u, e)
    op = bdda.Operator(n, lf, k)
    op.set_dipoles(addr)
    X, st = bdda.solve(op, diag, B, bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED, true_tol=1e-8,
                                                    itermax=3000), allow_not_converged=False)
    assert st["true_res_max"] <= 1e-8
    gh, P = mbt.green_hat(n, 3, lf, k)
    res = krylov.true_residual(lambda S: mbt.block_mvp(n, 3, gh, P, addr, diag, S), B, X)
    assert np.all(res < 2e-8), res


def test_server_accepts_box_sides_past_256():
    rng = np.random.default_rng(5)
    n = (330, 6, 4)
    N = int(np.prod(n))
    addr = np.sort(rng.choice(N, size=N // 3, replace=False)).astype(np.int32)
    wl0, m = 0.55, 1.5 + 0.1j
    k = 2 * np.pi / wl0
    lf = 0.5 / (abs(m) * k)
    alpha0 = bdda.polarizability(wl0, lf * (3 / (4 * np.pi)) ** (1 / 3), m * m, k)
    u, e = bdda.directions(1, 3)
    p = bdda.Problem(n=n, lf=lf, address=addr, k=k, alpha=np.full(addr.size, alpha0),
                     diag=np.full(3 * addr.size, 1.0 / alpha0), B=bdda.incident_fields(n, lf, addr, k, u, e))
    srv = bdda.Server(slots=2, mem_budget_bytes=20e9, opts=bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED,
                                                                           true_tol=1e-8, itermax=3000))
    X, r = srv.wait(srv.submit(p))
    srv.close()
    assert r["status"] == 0 and r["true_res_max"] <= 1e-8
    with pytest.raises(bdda.BddaError):
        big = bdda.Problem(n=(601, 2, 2), lf=lf, address=np.array([0], np.int32), k=k, alpha=np.array([alpha0]),
                           diag=np.full(3, 1.0 / alpha0), B=np.ones((3, 1), complex))
        srv2 = bdda.Server(slots=1, mem_budget_bytes=20e9, opts=bdda.solve_opts("cocg_rq", true_tol=1e-8))
        try:
            srv2.submit(big)
        finally:
            srv2.close()
