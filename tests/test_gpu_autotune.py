"""The FFT schedule autotuner (-m gpu): on an MVP large enough to be tuned
(FFT workspace >= 64 MiB) it times every candidate launch schedule of the
tile passes on the operator's own buffers and keeps the fastest; the tuned
MVP equals the default-schedule MVP (to FP32 rounding: the z-pass kernels
compute the same arithmetic from different memories), and the solve on the
tuned operator meets its true residual."""
import numpy as np
import pytest

import bdda

pytestmark = pytest.mark.gpu


def _mvp(op, x, L, n, diag):
    import torch
    xd = torch.from_numpy(np.ascontiguousarray(x.T)).to(torch.complex64).cuda()
    dd = torch.from_numpy(diag).to(torch.complex64).cuda()
    yd = torch.zeros_like(xd)
    torch.cuda.synchronize()
    op.mvp_device(xd.data_ptr(), yd.data_ptr(), L, n, n, prec=bdda.PREC_FP32, diag=dd.data_ptr(), jpre=dd.data_ptr())
    torch.cuda.synchronize()
    return yd.cpu().numpy().T.astype(np.complex128)


def test_autotuner_keeps_fastest_candidate_and_results():
    prob = bdda.make_problem(16384, 2.3 + 0.6j, seed=1, n_dirs=8)   # 144 x 160 x 150 grid, L = 16: 0.6 GB workspace
    L, n = 16, 3 * prob.nocc
    rng = np.random.default_rng(3)
    x = rng.standard_normal((n, L)) + 1j * rng.standard_normal((n, L))
    ref_op = bdda.Operator(prob.n, prob.lf, prob.k)
    ref_op.set_dipoles(prob.address)
    ref_op.set_autotune(False)
    y_def = _mvp(ref_op, x, L, n, prob.diag)
    sched_def, _, measured_def = ref_op.tuning(L)
    assert not measured_def and sched_def["y_waves"] == 4 and sched_def["y_buffers"] == 2
    op = bdda.Operator(prob.n, prob.lf, prob.k)
    op.set_dipoles(prob.address)
    y_tuned = _mvp(op, x, L, n, prob.diag)
    sched, cand, measured = op.tuning(L)
    assert measured
    ys = cand["y"]
    assert all(v > 0 for v in ys.values())
    best = min(ys, key=ys.get)
    assert best == f"buf{sched['y_buffers']}_waves{sched['y_waves']}"
    yd = cand["y_inverse"]
    assert all(v > 0 for v in yd.values())
    assert min(yd, key=yd.get) == f"buf{sched['y_inverse_buffers']}_waves{sched['y_inverse_waves']}"
    xs = cand["x_cta_per_sm"]
    assert str(sched["x_cta_per_sm"]) == min(xs, key=xs.get)
    z = {k: v for k, v in cand["z_pass"].items() if v > 0}
    # Pz = 150, plan 10 x 15 (no fused step): scalar, packed and pipelined kernels are the candidates, and the
    # default rule runs the packed one (three 8-warp CTAs of it fit)
    assert op.info()[0][2] == 150 and op.plans()["z"] == [10, 15]
    assert sorted(z) == ["packed", "pipelined", "scalar"]
    assert sched["z_pass"] == min(z, key=z.get)
    if sched["z_pass"] == "packed":
        assert np.array_equal(y_tuned, y_def)
    else:   # the packed kernel rounds its pair arithmetic differently
        assert np.linalg.norm(y_tuned - y_def) / np.linalg.norm(y_def) < 5e-6
    # the tuned schedule is kept: a second call gives the same bits
    assert np.array_equal(_mvp(op, x, L, n, prob.diag), y_tuned)
    # and a solve on the tuned operator still meets its true residual
    X, st = bdda.solve(op, prob.diag, prob.B, bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED, true_tol=1e-8,
                                                               itermax=3000), allow_not_converged=False)
    assert st["true_res_max"] <= 1e-8
