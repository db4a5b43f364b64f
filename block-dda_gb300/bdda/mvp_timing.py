"""Per-pass timing of the block MVP on a seeded aggregate (a sizing and profiling aid).

    python -m bdda.mvp_timing --nocc 65536 --nrhs 32 --m 1.78 [--reps 5] [--df]

Builds the operator of ``bdda.make_problem(nocc, m, seed=1)`` (the benchmark's
seeded aggregates), runs two warm complex FP32 block MVPs (the first one also
runs the FFT schedule autotuner where the workspace is large enough), then
``reps`` timed ones with every pass bracketed by CUDA events, and prints one
JSON line: grid, per-pass ms per launch, the algorithmic bytes of each pass
(``bdda_op_mvp_bytes``) and the autotuned schedule.  ``--df`` adds the
double-float MVP of the mixed solves' residuals.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np


def _to_df(a):
    hi_r = a.real.astype(np.float32)
    hi_i = a.imag.astype(np.float32)
    lo_r = (a.real - hi_r.astype(np.float64)).astype(np.float32)
    lo_i = (a.imag - hi_i.astype(np.float64)).astype(np.float32)
    return np.stack([hi_r, lo_r, hi_i, lo_i], axis=-1)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--nocc", type=int, default=65536)
    ap.add_argument("--nrhs", type=int, default=32)
    ap.add_argument("--m", default="1.78")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--df", action="store_true")
    a = ap.parse_args(argv)
    import torch
    import bdda
    prob = bdda.make_problem(a.nocc, complex(a.m), seed=1, n_dirs=max(1, a.nrhs // 2))
    L = a.nrhs
    op = bdda.Operator(prob.n, prob.lf, prob.k)
    op.set_dipoles(prob.address)
    n = 3 * prob.nocc
    B = prob.B[:, :L] if prob.B.shape[1] >= L else np.repeat(prob.B, L, axis=1)[:, :L]
    x = torch.from_numpy(np.ascontiguousarray(B.T)).to(torch.complex64).cuda()
    y = torch.zeros_like(x)
    d = torch.from_numpy(prob.diag).to(torch.complex64).cuda()

    def mvp32():
        op.mvp_device(x.data_ptr(), y.data_ptr(), L, n, n, prec=bdda.PREC_FP32, diag=d.data_ptr(), jpre=d.data_ptr())

    for _ in range(2):
        mvp32()
    torch.cuda.synchronize()
    op.set_timing(True)
    op.kernel_stats(reset=True)
    for _ in range(a.reps):
        mvp32()
    torch.cuda.synchronize()
    ks = op.kernel_stats(reset=True)
    if a.df:
        xdf = torch.from_numpy(np.ascontiguousarray(_to_df(B.T))).cuda()
        ydf = torch.zeros_like(xdf)
        ddf = torch.from_numpy(np.ascontiguousarray(_to_df(prob.diag))).cuda()
        for _ in range(1 + a.reps):
            op.mvp_device(xdf.data_ptr(), ydf.data_ptr(), L, n, n, prec=bdda.PREC_DF64, diag=ddf.data_ptr())
        torch.cuda.synchronize()
        kd = op.kernel_stats(reset=True)
        ks.update({k: v for k, v in kd.items() if k.endswith("c128") and v["launches"]})
    op.set_timing(False)
    sched, cand, measured = op.tuning(L)
    op.check_status()
    out = {"nocc": a.nocc, "nrhs": L, "box": list(prob.n), "grid": list(op.info()[0]), "plans": op.plans(),
           "ms_per_launch": {k: round(v["ms"] / max(1, v["launches"]), 4) for k, v in ks.items() if v["launches"]},
           "bytes": dict(zip("ABCDE", [float(v) for v in op.mvp_bytes(L, bdda.PREC_FP32, True, True)])),
           "schedule": sched, "autotuned": measured,
           "z_pass_candidates_ms": {k: round(v, 4) for k, v in cand["z_pass"].items() if v > 0}}
    op.close()
    print(json.dumps(out), flush=True)
    return 0


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.exit(main())
