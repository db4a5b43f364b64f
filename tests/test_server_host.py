"""Admission and queueing of the request server, on the CPU (dry-run executor,
no device work): memory budget never exceeded, oversize requests rejected,
every request completed once, large requests not starved by small ones."""
import numpy as np
import pytest

import bdda


def _probs(sizes, L=2, seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for i, n in enumerate(sizes):
        out.append(bdda.make_problem(int(n), 1.5 + 0.1j, seed=int(rng.integers(1, 10 ** 6)), n_dirs=max(1, L // 2)))
    return out


def test_footprint_grows_with_box_and_nrhs():
    a = bdda.footprint((20, 20, 20), 500, 2)
    b = bdda.footprint((40, 40, 40), 500, 2)
    c = bdda.footprint((40, 40, 40), 500, 16)
    assert 0 < a < b < c
    assert bdda.footprint((40, 40, 40), 500, 16, bdda.SOLVE_FP64) != c


def test_dry_run_respects_budget_and_completes_everything():
    probs = _probs([64, 300, 1000, 2500, 90, 700, 4000, 150, 2000, 80, 512, 3000], seed=1)
    fps = [bdda.footprint(p.n, p.nocc, p.B.shape[1]) for p in probs]
    budget = 2.2 * max(fps)
    opts = bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED, true_tol=1e-8)
    srv = bdda.Server(slots=4, mem_budget_bytes=budget, opts=opts, dry_run=True)
    tickets = [srv.submit(p) for p in probs]
    results = [srv.wait(t)[1] for t in tickets]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(probs)
    assert st["peak_inflight_bytes"] <= budget
    assert 2 <= st["peak_running"] <= 4
    for r, fp in zip(results, fps):
        assert r["status"] == 0 and r["t_submit"] <= r["t_start"] <= r["t_done"]
        assert abs(r["footprint_bytes"] - fp) < 1.0


def test_oversize_request_rejected():
    p = _probs([3000], seed=2)[0]
    opts = bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED, true_tol=1e-8)
    srv = bdda.Server(slots=2, mem_budget_bytes=0.5 * bdda.footprint(p.n, p.nocc, 2), opts=opts, dry_run=True)
    with pytest.raises(bdda.BddaError) as ei:
        srv.submit(p)
    assert ei.value.code == bdda.ERR_NOMEM
    srv.close()


def test_large_request_is_not_starved():
    small = _probs([64] * 40, seed=3)
    big = _probs([5000], seed=4)[0]
    fb = bdda.footprint(big.n, big.nocc, 2)
    fs = bdda.footprint(small[0].n, small[0].nocc, 2)
    budget = fb + 0.5 * fs          # the big one only fits when nothing else runs
    opts = bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED, true_tol=1e-8)
    srv = bdda.Server(slots=4, mem_budget_bytes=budget, opts=opts, dry_run=True)
    t_small1 = [srv.submit(p) for p in small[:4]]
    t_big = srv.submit(big)
    t_small2 = [srv.submit(p) for p in small[4:]]
    r_big = srv.wait(t_big)[1]
    later = [srv.wait(t)[1] for t in t_small2]
    [srv.wait(t) for t in t_small1]
    srv.close()
    # at most 8 later requests may overtake the waiting big one
    overtook = sum(1 for r in later if r["t_start"] < r_big["t_start"])
    assert overtook <= 8


def test_server_requires_true_residual_mode():
    with pytest.raises(bdda.BddaError):
        bdda.Server(slots=1, mem_budget_bytes=1e9, opts=bdda.solve_opts(true_tol=0.0), dry_run=True)
