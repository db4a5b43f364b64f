"""f = 6 (electric + magnetic dipoles, the reference's CEMD mode) on the GPU (-m gpu).

* MBT_fft_mvp on the cuboid vector vs the literal 1-D MBT restatement (FP64);
* the block MVP (diag, Jacobi) in FP64, complex FP32 and double-float vs the
  oracle's 3-D padded FFT with the 6x6 block [[-G, -F], [F, -G]];
* the recorded BiCGSTAB-Jacobi runs of DDA_result_BC_rpp20nm.dat (tol 1e-2,
  4 incident waves, N8..N64 targets at eleven wavelengths) reproduced through
  the C ABI: to the printed digits where the run is short and Csca is not a
  small difference, MAC to 1e-3 everywhere;
* mixed-precision refinement to a true residual of 1e-8 agrees with FP64.
"""
import math

import numpy as np
import pytest

import bdda
from conftest import golden
from oracle import mbt, physics

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 5e-6


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("n", [(3, 2, 4), (2, 3, 2), (4, 3, 3)])
def test_f6_mbt_fft_mvp_matches_literal_reference(n):
    rng = np.random.default_rng(sum(n) + 6)
    lf, k = 0.29, 1.7 + 0.03j
    N = int(np.prod(n))
    x = rng.standard_normal(6 * N) + 1j * rng.standard_normal(6 * N)
    ref = mbt.mbt_fft_mvp(n, 6, mbt.mbt_fft_init(n, 6, lf, k), x)
    op = bdda.Operator(n, lf, k, prec=bdda.PREC_FP64, f=6)
    assert _rel(op.mbt_fft_mvp(x), ref) < TOL64


@pytest.mark.parametrize("nocc,L", [(2, 1), (57, 3), (300, 4), (1200, 2)])
def test_f6_block_mvp_vs_oracle(nocc, L):
    import torch
    n, addr = bdda.aggregate(nocc, 1.0, 2.8, 40 + nocc)
    rng = np.random.default_rng(nocc)
    x = rng.standard_normal((6 * nocc, L)) + 1j * rng.standard_normal((6 * nocc, L))
    diag = rng.standard_normal(6 * nocc) + 1j * rng.standard_normal(6 * nocc) + 5.0
    jpre = 1.0 / diag
    lf, k = 0.021, 2 * np.pi / 0.55
    gh, P = mbt.green_hat(n, 6, lf, k)
    ref = mbt.block_mvp(n, 6, gh, P, addr, diag, x, jpre)
    op = bdda.Operator(n, lf, k, f=6)
    op.set_dipoles(addr)
    for prec, dt, tol in ((bdda.PREC_FP64, torch.complex128, TOL64), (bdda.PREC_FP32, torch.complex64, TOL32)):
        xd = torch.from_numpy(np.ascontiguousarray(x.T)).to(dt).cuda()
        yd = torch.zeros_like(xd)
        dd = torch.from_numpy(diag).to(dt).cuda()
        jd = torch.from_numpy(jpre).to(dt).cuda()
        torch.cuda.synchronize()
        op.mvp_device(xd.data_ptr(), yd.data_ptr(), L, 6 * nocc, 6 * nocc, prec=prec, diag=dd.data_ptr(),
                      jpre=jd.data_ptr())
        torch.cuda.synchronize()
        assert _rel(yd.cpu().numpy().T, ref) < tol, prec

    def to_df(a):   # complex128 -> float32 [..., 4] = (re_hi, re_lo, im_hi, im_lo)
        hr, hi = a.real.astype(np.float32), a.imag.astype(np.float32)
        return np.stack([hr, (a.real - hr).astype(np.float32), hi, (a.imag - hi).astype(np.float32)], axis=-1)

    ref0 = mbt.block_mvp(n, 6, gh, P, addr, diag, x)
    xd = torch.from_numpy(np.ascontiguousarray(to_df(x.T))).cuda()
    dd = torch.from_numpy(np.ascontiguousarray(to_df(diag))).cuda()
    yd = torch.zeros_like(xd)
    torch.cuda.synchronize()
    op.mvp_device(xd.data_ptr(), yd.data_ptr(), L, 6 * nocc, 6 * nocc, prec=bdda.PREC_DF64, diag=dd.data_ptr())
    torch.cuda.synchronize()
    y = yd.cpu().numpy().astype(np.float64)
    got = ((y[..., 0] + y[..., 1]) + 1j * (y[..., 2] + y[..., 3])).T
    assert _rel(got, ref0) < TOL64


def _f6_case(g, c):
    t = g["targets"][c["target"]]
    s = g["scale_factor"]
    n, lf, addr = tuple(t["n"]), t["lf"] * s, np.array(t["address"])
    k = 2 * math.pi / c["wl0"]
    ae, ah = complex(*c["alpha_e0"]), complex(*c["alpha_h0"])
    nocc = addr.size
    diag = bdda.diag_a(np.full(nocc, ae), np.full(nocc, ah))
    u, e, h = physics.reference_incident_waves(4)
    B = bdda.incident_fields(n, lf, addr, k, u, e, h)
    return n, lf, addr, k, ae, ah, diag, B


def test_f6_recorded_runs_reproduced_on_gpu():
    g = golden("result_f6_BC_rpp20nm.json")
    nstrict = 0
    for c in g["cases"]:
        n, lf, addr, k, ae, ah, diag, B = _f6_case(g, c)
        op = bdda.Operator(n, lf, k, prec=bdda.PREC_FP64, f=6)
        op.set_dipoles(addr)
        X, st = bdda.solve(op, diag, B, bdda.solve_opts("bicgstab", jacobi=True, tol=g["tol"], itermax=g["itermax"]))
        cext, cabs, csca = bdda.cross_sections(k, ae, B, X, ah)
        rec = c["recorded"]
        mac = (cabs * 1e-12 / rec["mass_particle"]).mean()
        assert abs(mac - rec["mean_MAC"]) / rec["mean_MAC"] < 1e-3, (c["target"], c["wl0"])
        if c["oracle_iterations"] <= 8 and rec["mean_SSA"] > 0.05:
            nstrict += 1
            assert st["iterations"] == c["oracle_iterations"], (c["target"], c["wl0"])
            for got, key in ((csca.mean(), "mean_Csca"), (mac, "mean_MAC"), ((csca / cext).mean(), "mean_SSA")):
                assert abs(got - rec[key]) / abs(rec[key]) < 6e-6, (c["target"], c["wl0"], key, got, rec[key])
        op.close()
    assert nstrict >= 15


@pytest.mark.parametrize("solver", ["bicgstab", "cocg_rq"])
def test_f6_mixed_refinement_matches_fp64(solver):
    nocc, L = 900, 6
    n, addr = bdda.aggregate(nocc, 1.0, 2.8, 17)
    wl0, m = 0.55, 1.9 + 0.4j
    k = 2 * math.pi / wl0
    lf = 0.5 / (abs(m) * k)
    r_eq = lf * (3 / (4 * math.pi)) ** (1 / 3)
    ae, ah = bdda.polarizabilities(wl0, r_eq, m * m, k)
    diag = bdda.diag_a(np.full(nocc, ae), np.full(nocc, ah))
    u, e, h = physics.reference_incident_waves(L)
    B = bdda.incident_fields(n, lf, addr, k, u, e, h)
    op = bdda.Operator(n, lf, k, f=6)
    op.set_dipoles(addr)
    res = {}
    for prec in (bdda.SOLVE_FP64, bdda.SOLVE_MIXED):
        X, st = bdda.solve(op, diag, B, bdda.solve_opts(solver, jacobi=True, precision=prec, true_tol=1e-8,
                                                         itermax=2000), allow_not_converged=False)
        assert st["true_res_max"] <= 1e-8
        res[prec] = bdda.cross_sections(k, ae, B, X, ah)
    for a, b in zip(res[bdda.SOLVE_FP64], res[bdda.SOLVE_MIXED]):
        assert np.max(np.abs(a - b) / np.abs(b)) < 1e-6
