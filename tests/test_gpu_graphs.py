"""Poll cycles of the block Krylov solvers as captured CUDA graphs (-m gpu).

Every solve runs its first poll cycle launch by launch and each later
cycle (check_every iterations between two reads of the control block) as one
launch of a captured graph; BDDA_NO_GRAPH=1 turns the graphs off.  A graph
holds the same kernels in the same order with the same arguments, so a solve
gives bitwise the same solution, iteration count and per-class launch counts
either way, and the timed fused z pass keeps its CUDA-event time inside the
graph.  A cached graph is not replayed after the operator's dipoles changed,
and bdda_op_set_graphs switches the graphs per operator.
"""
import os

import numpy as np
import pytest

import bdda
from oracle import krylov, mbt

pytestmark = pytest.mark.gpu


def _solve(op, diag, B, opts, graphs):
    if graphs:
        os.environ.pop("BDDA_NO_GRAPH", None)
    else:
        os.environ["BDDA_NO_GRAPH"] = "1"
    try:
        op.kernel_stats(reset=True)
        X, st = bdda.solve(op, diag, B, opts, allow_not_converged=False)
        return X, st, op.kernel_stats()
    finally:
        os.environ.pop("BDDA_NO_GRAPH", None)


@pytest.mark.parametrize("solver", ["cocg_rq", "bicgstab", "bicggr"])
@pytest.mark.parametrize("precision", [bdda.SOLVE_FP64, bdda.SOLVE_MIXED])
@pytest.mark.parametrize("timing", [0, 2])
def test_graph_cycles_match_direct_launches(solver, precision, timing):
    prob = bdda.make_problem(1024, 1.95 + 0.79j, seed=1, n_dirs=2)
    op = bdda.Operator(prob.n, prob.lf, prob.k)
    op.set_dipoles(prob.address)
    op.set_timing(timing)
    opts = bdda.solve_opts(solver, jacobi=True, precision=precision, true_tol=1e-8, itermax=1000)
    Xd, sd, kd = _solve(op, prob.diag, prob.B, opts, graphs=False)
    Xg, sg, kg = _solve(op, prob.diag, prob.B, opts, graphs=True)   # captures the cycle
    Xr, sr, kr = _solve(op, prob.diag, prob.B, opts, graphs=True)   # replays the cached one
    assert sd["iterations"] > 8  # at least one cycle ran as a graph
    for s in (sg, sr):
        assert s["iterations"] == sd["iterations"] and s["status"] == 0
        assert s["true_res_max"] == sd["true_res_max"] and s["mvps"] == sd["mvps"]
    assert np.array_equal(Xg, Xd) and np.array_equal(Xr, Xd)
    for name in kd:
        assert kg[name]["launches"] == kd[name]["launches"] == kr[name]["launches"], name
    if timing == 2:
        timed = "passC_c128" if precision == bdda.SOLVE_FP64 else "passC_c64"
        for k in (kg, kr):
            assert k[timed]["ms"] > 0.0
            assert 0.5 < k[timed]["ms"] / kd[timed]["ms"] < 2.0, (k[timed]["ms"], kd[timed]["ms"])


def test_graph_not_replayed_after_dipoles_change():
    """Same box, same dipole count, other sites: the occupied tiles differ, and
    the operator reused after set_dipoles gives bitwise the solution of a
    fresh operator on the new sites."""
    prob = bdda.make_problem(900, 1.7 + 0.3j, seed=3, n_dirs=2)
    rng = np.random.default_rng(5)
    nsite = int(np.prod(prob.n))
    other = np.sort(rng.choice(nsite, size=len(prob.address), replace=False)).astype(np.int32)
    assert not np.array_equal(other, prob.address)
    opts = bdda.solve_opts("cocg_rq", jacobi=True, precision=bdda.SOLVE_MIXED, true_tol=1e-8, itermax=2000)
    reused = bdda.Operator(prob.n, prob.lf, prob.k)
    reused.set_dipoles(prob.address)
    _solve(reused, prob.diag, prob.B, opts, graphs=True)
    reused.set_dipoles(other)
    Xu, su, _ = _solve(reused, prob.diag, prob.B, opts, graphs=True)
    fresh = bdda.Operator(prob.n, prob.lf, prob.k)
    fresh.set_dipoles(other)
    Xf, sf, _ = _solve(fresh, prob.diag, prob.B, opts, graphs=True)
    assert su["iterations"] == sf["iterations"]
    assert np.array_equal(Xu, Xf)
    gh, P = mbt.green_hat(prob.n, 3, prob.lf, prob.k)
    amul = lambda S: mbt.block_mvp(prob.n, 3, gh, P, other, prob.diag, S)  # noqa: E731
    assert np.all(krylov.true_residual(amul, prob.B, Xu) < 2e-8)


def test_set_graphs_switch():
    """bdda_op_set_graphs(op, 0) runs the same solve launch by launch: bitwise
    the same solution and the same launch counts as with the graphs."""
    prob = bdda.make_problem(1024, 1.95 + 0.79j, seed=2, n_dirs=2)
    op = bdda.Operator(prob.n, prob.lf, prob.k)
    op.set_dipoles(prob.address)
    opts = bdda.solve_opts("cocg_rq", jacobi=True, precision=bdda.SOLVE_MIXED, true_tol=1e-8, itermax=1000)
    out = {}
    for on in (False, True, False):
        op.set_graphs(on)
        op.kernel_stats(reset=True)
        X, st = bdda.solve(op, prob.diag, prob.B, opts, allow_not_converged=False)
        out.setdefault(on, []).append((X, st, op.kernel_stats()))
    Xd, sd, kd = out[False][0]
    for X, st, k in out[True] + out[False][1:]:
        assert np.array_equal(X, Xd) and st["iterations"] == sd["iterations"] and st["mvps"] == sd["mvps"]
        assert all(k[name]["launches"] == kd[name]["launches"] for name in kd)
