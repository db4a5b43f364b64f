"""Block Krylov solvers on the GPU against the oracle (parity tests, -m gpu).

* reference semantics (one solve, the reference's recurrence error and tol):
  same iteration count as the oracle restatement, per-iteration errors within
  1e-6 relative, solution within 1e-6 relative;
* the recorded run result.dat (f=3 block COCG-RQ-Jacobi, N512 target, tol 1e-2)
  reproduced through the C ABI to its printed digits;
* refinement mode: every column's true residual <= 1e-8, FP64 and mixed
  precision; the mixed solve's cross sections and polarisation within 1e-6 of
  the oracle's FP64 block COCG-RQ-Jacobi solve.
"""
import math

import numpy as np
import pytest

import bdda
from conftest import golden
from oracle import krylov, mbt, physics, torch3d

pytestmark = pytest.mark.gpu


def _small_problem(nocc=150, L=4, seed=21, m=1.7 + 0.3j):
    prob = bdda.make_problem(nocc, m, seed=seed, n_dirs=max(1, L // 2))
    rng = np.random.default_rng(seed)
    B = prob.B[:, :L]
    if B.shape[1] < L:
        B = np.concatenate([B, rng.standard_normal((B.shape[0], L - B.shape[1]))], axis=1)
    return prob, np.asfortranarray(B)


def _oracle_amul(prob):
    gh, P = mbt.green_hat(prob.n, 3, prob.lf, prob.k)
    return lambda S: mbt.block_mvp(prob.n, 3, gh, P, prob.address, prob.diag, S)


def test_qr_reduced_matches_oracle():
    rng = np.random.default_rng(2)
    for m, n in ((40, 1), (300, 7), (1000, 32)):
        a = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
        q, r = bdda.qr_reduced(a)
        qo, ro = krylov.qr_reduced(a)
        assert np.max(np.abs(q - qo)) < 1e-12
        assert np.max(np.abs(r - ro)) / np.max(np.abs(ro)) < 1e-13


@pytest.mark.parametrize("solver", ["cocg_rq", "bicgstab", "bicggr"])
@pytest.mark.parametrize("jacobi", [False, True])
def test_solver_reference_semantics_vs_oracle(solver, jacobi):
    prob, B = _small_problem()
    amul = _oracle_amul(prob)
    Xo, hist = krylov.SOLVERS[solver](amul, B, 1e-6, 300, diag=prob.diag, jacobi=jacobi)
    op = bdda.Operator(prob.n, prob.lf, prob.k)
    op.set_dipoles(prob.address)
    opts = bdda.solve_opts(solver=solver, jacobi=jacobi, tol=1e-6, itermax=300)
    X, st = bdda.solve(op, prob.diag, B, opts)
    assert st["status"] == 0
    assert st["iterations"] == len(hist), (st["iterations"], len(hist))
    assert abs(st["final_err"] - hist[-1]) / hist[-1] < 1e-4
    assert np.linalg.norm(X - Xo) / np.linalg.norm(Xo) < 1e-6


def test_result_dat_reproduced_on_gpu():
    t = golden("target_N512.json")
    g = golden("result_dat_N512.json")
    scale = g["scale_factor"]
    n = tuple(t["n"])
    lf = t["lf"] * scale
    addr = np.array(t["address"], dtype=np.int32)
    vol = np.array(t["vol"]) * scale ** 3
    k = 2 * math.pi / 0.3
    r_p = np.cbrt(3 * vol / (4 * math.pi))
    alpha = np.array([bdda.polarizability(0.3, r, complex(*g["eper"]), k) for r in r_p])
    diag = np.repeat(1.0 / alpha, 3)
    u, e, _ = physics.reference_incident_waves(4)
    B = bdda.incident_fields(n, lf, addr, k, u, e)
    op = bdda.Operator(n, lf, k)
    op.set_dipoles(addr)
    X, st = bdda.solve(op, diag, B, bdda.solve_opts("cocg_rq", jacobi=True, tol=1e-2, itermax=300))
    assert st["iterations"] == len(g["oracle_history"])
    cext, cabs, csca = bdda.cross_sections(k, alpha[0], B, X)
    rec = g["recorded"]
    mass = vol.sum() * 1e-12 * g["density"]
    assert abs(csca.mean() - rec["mean_Csca"]) / rec["mean_Csca"] < 2e-6
    assert abs(csca.std(ddof=1) - rec["std_Csca"]) / rec["std_Csca"] < 2e-5
    assert abs((cabs * 1e-12 / mass).mean() - rec["mean_MAC"]) / rec["mean_MAC"] < 2e-6
    assert abs((csca / cext).mean() - rec["mean_SSA"]) / rec["mean_SSA"] < 2e-6
    assert np.allclose(csca, g["oracle_Csca"], rtol=1e-7)


@pytest.mark.parametrize("precision", [bdda.SOLVE_FP64, bdda.SOLVE_MIXED])
@pytest.mark.parametrize("solver", ["cocg_rq", "bicgstab"])
def test_refinement_reaches_true_residual(precision, solver):
    prob = bdda.make_problem(1024, 1.95 + 0.79j, seed=1, n_dirs=1)
    op = bdda.Operator(prob.n, prob.lf, prob.k)
    op.set_dipoles(prob.address)
    opts = bdda.solve_opts(solver, jacobi=True, precision=precision, true_tol=1e-8, itermax=1000)
    X, st = bdda.solve(op, prob.diag, prob.B, opts, allow_not_converged=False)
    assert st["true_res_max"] <= 1e-8
    res = krylov.true_residual(_oracle_amul(prob), prob.B, X)
    assert np.all(res < 2e-8), res


def test_mixed_solve_matches_oracle_solve_N2000():
    """Mixed GPU solve against the oracle's block COCG-RQ-Jacobi (FP64, run to a
    recurrence error of 1e-11) on the torch operator: cross sections and
    polarisation within 1e-6."""
    prob = bdda.make_problem(2000, 2.3 + 0.6j, seed=4, n_dirs=4)
    ind = torch3d.GreenOperator(prob.n, prob.lf, prob.k, prob.address, device="cuda")

    def amul(S):
        return prob.diag[:, None] * S + ind.apply(S).cpu().numpy()

    Xo, _hist = krylov.bl_cocg_rq(amul, prob.B, 1e-11, 1000, diag=prob.diag, jacobi=True)
    assert np.all(krylov.true_residual(amul, prob.B, Xo) <= 1e-10)
    op = bdda.Operator(prob.n, prob.lf, prob.k)
    op.set_dipoles(prob.address)
    X, st = bdda.solve(op, prob.diag, prob.B, bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED,
                                                                true_tol=1e-8, itermax=2000),
                       allow_not_converged=False)
    assert st["true_res_max"] <= 1e-8
    cg = bdda.cross_sections(prob.k, prob.alpha[0], prob.B, X)
    co = bdda.cross_sections(prob.k, prob.alpha[0], prob.B, Xo)
    for a, b in zip(cg, co):
        assert np.max(np.abs(a - b) / np.abs(b)) < 1e-6
    assert np.linalg.norm(X - Xo) / np.linalg.norm(Xo) < 1e-6


def test_mixed_solve_on_fp32_and_double_float_tables_only():
    """An operator holding only the tables a mixed solve uses (FP32 inner
    solves, double-float true residuals) gives the same solution as one with
    every table; an FP64 solve on it is refused."""
    prob = bdda.make_problem(1500, 2.3 + 0.6j, seed=6, n_dirs=2)
    opts = bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED, true_tol=1e-8, itermax=2000)
    full = bdda.Operator(prob.n, prob.lf, prob.k)
    full.set_dipoles(prob.address)
    lean = bdda.Operator(prob.n, prob.lf, prob.k, prec=bdda.PREC_FP32 | bdda.PREC_DF64)
    lean.set_dipoles(prob.address)
    Xf, sf = bdda.solve(full, prob.diag, prob.B, opts, allow_not_converged=False)
    Xl, sl = bdda.solve(lean, prob.diag, prob.B, opts, allow_not_converged=False)
    assert sl["true_res_max"] <= 1e-8 and sl["iterations"] == sf["iterations"]
    assert np.array_equal(Xl, Xf)  # same tables, same kernels, same order: bitwise
    res = krylov.true_residual(_oracle_amul(prob), prob.B, Xl)
    assert np.all(res < 2e-8), res
    with pytest.raises(bdda.BddaError):
        bdda.solve(lean, prob.diag, prob.B, bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_FP64, true_tol=1e-8))


def test_mixed_refinement_with_unequal_residual_columns():
    """A case of the serving stream (N=17523, L=32, m=2.11+0.23i,
    lambda=0.398 um) whose residual after the first refinement step has
    columns of very different sizes: the FP32 Gram of that block loses positive
    definiteness unless the inner right-hand side is scaled to unit columns
    (CholQR broke down there).  It must converge."""
    prob = bdda.make_problem(17523, 2.1095600183974708 + 0.22780528458440563j, wl0=0.3976663593698059,
                             kf=1.0931588914517667, Df=2.718068505948526, seed=940342375, n_dirs=16)
    assert prob.B.shape[1] == 32
    op = bdda.Operator(prob.n, prob.lf, prob.k)
    op.set_dipoles(prob.address)
    opts = bdda.solve_opts("cocg_rq", jacobi=True, precision=bdda.SOLVE_MIXED, true_tol=1e-8, itermax=3000)
    _X, st = bdda.solve(op, prob.diag, prob.B, opts, allow_not_converged=False)
    assert st["status"] == 0 and st["true_res_max"] <= 1e-8


def test_solve_status_codes():
    prob, B = _small_problem(nocc=60, L=2)
    op = bdda.Operator(prob.n, prob.lf, prob.k)
    op.set_dipoles(prob.address)
    _X, st = bdda.solve(op, prob.diag, B, bdda.solve_opts("cocg_rq", tol=1e-14, itermax=3))
    assert st["status"] == bdda.ERR_NOT_CONVERGED and st["iterations"] == 3
    Bz = B.copy()
    Bz[:, 1] = 0.0
    with pytest.raises(bdda.BddaError) as ei:
        bdda.solve(op, prob.diag, Bz, bdda.solve_opts("cocg_rq", true_tol=1e-8))
    assert ei.value.code == bdda.ERR_INVALID
    with pytest.raises(bdda.BddaError):
        bdda.solve(op, prob.diag, np.zeros((3 * prob.nocc, 33)), bdda.solve_opts())


def test_mixed_solve_falls_back_to_fp64_inner_solves():
    """The reference's N1024 aggregate with its own site volumes (spheres of
    radius d on a lattice of spacing d) at m = 1.78 is so ill-conditioned that
    FP32 Krylov stagnates (FP64 COCG-RQ needs ~350 iterations); the mixed
    refinement must switch to FP64 inner solves and still reach the true
    residual, with the FP64 solve's cross sections."""
    import os
    from conftest import GOLDEN
    d = np.load(os.path.join(GOLDEN, "target_N1024.npz"))
    addr = np.cumsum(d["address_delta"].astype(np.int64)).astype(np.int32)
    n = tuple(int(v) for v in d["n"])
    prob = bdda.target_problem(n, float(d["lf"]), addr, float(d["vol"]), 1.78, wl0=0.55, seed=1, n_dirs=4)
    op = bdda.Operator(prob.n, prob.lf, prob.k)
    op.set_dipoles(prob.address)
    X64, s64 = bdda.solve(op, prob.diag, prob.B, bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_FP64, true_tol=1e-8,
                                                                  itermax=3000), allow_not_converged=False)
    Xm, sm = bdda.solve(op, prob.diag, prob.B, bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED, true_tol=1e-8,
                                                                itermax=3000), allow_not_converged=False)
    assert s64["iterations"] > 200
    assert sm["status"] == 0 and sm["true_res_max"] <= 1e-8 and sm["fp64_inner_steps"] >= 1
    res = krylov.true_residual(_oracle_amul(prob), prob.B, Xm)
    assert np.all(res < 2e-8), res
    cm = bdda.cross_sections(prob.k, prob.alpha[0], prob.B, Xm)
    c64 = bdda.cross_sections(prob.k, prob.alpha[0], prob.B, X64)
    for a, b in (cm[0], c64[0]), (cm[2], c64[2]):  # Cext, Csca (real m: Cabs is rounding noise)
        assert np.max(np.abs(a - b) / np.abs(b)) < 1e-6
