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


def test_server_takes_f6_requests():
    """An f = 6 (electric + magnetic dipole) request through the server equals
    the direct solve on an f = 6 operator with the server's tables (FP32 +
    double-float) bitwise, next to f = 3 requests in the same mix."""
    import math
    from oracle import physics
    nocc, L = 700, 4
    n, addr = bdda.aggregate(nocc, 1.0, 2.8, 29)
    wl0, m = 0.55, 1.9 + 0.4j
    k = 2 * math.pi / wl0
    lf = 0.5 / (abs(m) * k)
    ae, ah = bdda.polarizabilities(wl0, lf * (3 / (4 * math.pi)) ** (1 / 3), m * m, k)
    diag = bdda.diag_a(np.full(nocc, ae), np.full(nocc, ah))
    u, e, h = physics.reference_incident_waves(L)
    B = bdda.incident_fields(n, lf, addr, k, u, e, h)
    p6 = bdda.Problem(n=n, lf=lf, address=addr, k=k, alpha=np.full(nocc, ae), diag=diag, B=B)
    opts = _mixed_opts()
    op = bdda.Operator(n, lf, k, prec=bdda.PREC_FP32 | bdda.PREC_DF64, f=6)
    op.set_dipoles(addr)
    op.set_graphs(False)
    X_direct, st = bdda.solve(op, diag, B, opts, allow_not_converged=False)
    op.close()
    assert bdda.footprint(n, nocc, L, f=6) > bdda.footprint(n, nocc, L, f=3)
    srv = bdda.Server(slots=3, mem_budget_bytes=20e9, opts=opts)
    others = _problems(3, 31)
    tickets = [srv.submit(others[0]), srv.submit(p6)] + [srv.submit(p) for p in others[1:]]
    outs = {t: srv.wait(t) for t in tickets}
    srv.close()
    X6, r6 = outs[tickets[1]]
    assert r6["status"] == 0 and r6["true_res_max"] <= 1e-8
    assert X6.shape == (6 * nocc, L) and np.array_equal(X6, X_direct)
    assert all(outs[t][1]["status"] == 0 for t in tickets)


def test_server_reuses_cached_spectrum_bitwise():
    """A request with the box, spacing and wavenumber of a finished one takes
    its idle operator (Green spectra kept in HBM) instead of rebuilding it; the
    solution is bitwise the one of a fresh operator.  A different wavelength
    builds a new spectrum; with the cache off nothing is reused."""
    import dataclasses
    p = bdda.make_problem(900, 1.9 + 0.3j, seed=41, n_dirs=2)
    q = bdda.make_problem(900, 1.9 + 0.3j, wl0=0.6, seed=41, n_dirs=2)
    p2 = dataclasses.replace(p, B=np.asfortranarray(p.B[:, ::-1]))  # same target, other right-hand sides
    opts = _mixed_opts()
    srv = bdda.Server(slots=1, mem_budget_bytes=20e9, opts=opts)
    outs = [srv.wait(srv.submit(x)) for x in (p, q, p2, p)]
    st = srv.stats()
    srv.close()
    assert all(r["status"] == 0 for _, r in outs)
    assert st["spectra_built"] == 2 and st["spectra_reused"] == 2
    assert np.array_equal(outs[3][0], outs[0][0])
    fresh = bdda.Server(slots=1, mem_budget_bytes=20e9, opts=opts)
    fresh.set_spectrum_cache(0)
    X2, _ = fresh.wait(fresh.submit(p2))
    st0 = fresh.stats()
    fresh.close()
    assert st0["spectra_reused"] == 0 and st0["cached_bytes"] == 0
    assert np.array_equal(outs[2][0], X2)


def test_server_express_slot_serves_small_request_past_large_ones():
    """With the one regular slot busy with large requests (footprint > 2 GB),
    a small request submitted after them runs on an express slot and finishes
    first; every result still converges."""
    big = [bdda.make_problem(16384, 2.0 + 0.3j, seed=s, n_dirs=8) for s in (3, 4, 5)]
    small = bdda.make_problem(300, 1.5 + 0.1j, seed=3, n_dirs=1)
    assert all(bdda.footprint(p.n, p.nocc, 16) > 2e9 for p in big)
    assert bdda.footprint(small.n, small.nocc, 2) < 2e9
    srv = bdda.Server(slots=1, mem_budget_bytes=60e9, opts=_mixed_opts())
    tb = [srv.submit(p) for p in big]
    ts = srv.submit(small)
    rs = srv.wait(ts)[1]
    rb = [srv.wait(t)[1] for t in tb]
    st = srv.stats()
    srv.close()
    assert rs["status"] == 0 and all(r["status"] == 0 for r in rb)
    assert rs["t_done"] < max(r["t_done"] for r in rb)
    assert rs["t_done"] < rb[1]["t_start"] or rs["t_done"] < rb[0]["t_done"]
    assert st["peak_running"] >= 2
