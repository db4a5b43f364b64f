"""Bounded waits of the pipelined z pass (-m gpu).

The pipelined z pass waits on mbarriers for its bulk copies; every wait gives
up after 2 s, sets the operator's status word and lets the kernel return.  The
test hook bdda_op_test_z_stall makes one warp wait on a barrier that nothing
arrives on (no fault, no hang): the launch must return within a few seconds,
the status must be reported as an error, and the context must stay usable --
the next MVP gives the same bits as before.
"""
import time

import numpy as np
import pytest

import bdda

pytestmark = pytest.mark.gpu


def _mvp32(op, x, L, n):
    import torch
    xd = torch.from_numpy(np.ascontiguousarray(x.T)).to(torch.complex64).cuda()
    yd = torch.zeros_like(xd)
    torch.cuda.synchronize()
    op.mvp_device(xd.data_ptr(), yd.data_ptr(), L, n, n, prec=bdda.PREC_FP32)
    torch.cuda.synchronize()
    return yd.cpu().numpy().T.copy()


def test_pipelined_z_pass_wait_gives_up_and_is_reported():
    rng = np.random.default_rng(21)
    box = (6, 5, 120)                      # Pz = 240: two-stage fused z plan
    N = int(np.prod(box))
    nocc = N // 2
    addr = np.sort(rng.choice(N, size=nocc, replace=False)).astype(np.int32)
    L, n = 8, 3 * nocc
    x = rng.standard_normal((n, L)) + 1j * rng.standard_normal((n, L))
    op = bdda.Operator(box, 0.03, 2 * np.pi / 0.55)
    op.set_dipoles(addr)
    op.set_autotune(False)
    op.set_z_kernel("pipelined")
    y_ok = _mvp32(op, x, L, n)
    op.check_status()
    op.test_z_stall(True)
    t0 = time.monotonic()
    _mvp32(op, x, L, n)
    dt = time.monotonic() - t0
    with pytest.raises(bdda.BddaError) as err:
        op.check_status()
    assert err.value.code == bdda.ERR_CUDA and "gave up" in str(err.value)
    assert 1.5 < dt < 30.0, dt
    op.test_z_stall(False)
    op.check_status()                      # the word was cleared when read
    assert np.array_equal(_mvp32(op, x, L, n), y_ok)
    op.check_status()
    op.close()
