"""Batched solves and the request server on the GPU: every request reaches a
1e-8 true residual, and its solution is bitwise the same solved alone and
solved concurrently among other requests (-m gpu)."""
import numpy as np
import pytest

import bdda
from oracle import krylov, mbt

pytestmark = pytest.mark.gpu


def _mixed_opts():
    return bdda.solve_opts("cocg_rq", jacobi=True, precision=bdda.SOLVE_MIXED, true_tol=1e-8, itermax=3000)


def _problems(count, seed):
    rng = np.random.default_rng(seed)
    return [bdda.random_problem(rng, n_range=(64, 1500)) for _ in range(count)]


def test_batch_matches_single_solves_bitwise():
    probs = _problems(6, 11)
    opts = _mixed_opts()
    alone = []
    for p in probs:
        op = bdda.Operator(p.n, p.lf, p.k)
        op.set_dipoles(p.address)
        X, st = bdda.solve(op, p.diag, p.B, opts, allow_not_converged=False)
        alone.append(X)
        op.close()
    out = bdda.batch_solve(probs, slots=4, mem_budget_bytes=20e9, opts=opts)
    for (X, r), Xa, p in zip(out, alone, probs):
        assert r["status"] == 0 and r["true_res_max"] <= 1e-8
        assert np.array_equal(X, Xa)
    # and against the oracle's true residual for one of them
    p = probs[0]
    gh, P = mbt.green_hat(p.n, 3, p.lf, p.k)
    res = krylov.true_residual(lambda S: mbt.block_mvp(p.n, 3, gh, P, p.address, p.diag, S), p.B, out[0][0])
    assert np.all(res < 2e-8)


def test_server_result_same_alone_and_in_the_mix():
    probs = _problems(8, 23)
    opts = _mixed_opts()
    srv1 = bdda.Server(slots=1, mem_budget_bytes=20e9, opts=opts)
    X_alone, _ = srv1.wait(srv1.submit(probs[0]))
    srv1.close()
    srv = bdda.Server(slots=4, mem_budget_bytes=20e9, opts=opts)
    tickets = [srv.submit(p) for p in probs[1:4]] + [srv.submit(probs[0])] + [srv.submit(p) for p in probs[4:]]
    outs = {t: srv.wait(t) for t in tickets}
    st = srv.stats()
    srv.close()
    X_mix, r = outs[tickets[3]]
    assert r["status"] == 0
    assert np.array_equal(X_mix, X_alone)
    assert st["completed"] == len(probs) and st["peak_running"] >= 2
