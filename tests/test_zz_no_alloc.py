"""The allocation-free block MVP (bdda_op_mvp_device_noalloc).

It serves callers that cannot let the library allocate device memory: hosts
that own all GPU memory through their own pool, and serving loops that must not
enter the CUDA allocator.  Its result must equal the regular (allocating) entry
point's, call after call, while its scratch is the library's fixed device array.
This file sorts last so a run that stops at the first failure has run every
other test first; it also passes when run alone in a fresh process.
"""
import numpy as np
import pytest

import bdda

pytestmark = pytest.mark.gpu

TOL = {bdda.PREC_FP64: 1e-12, bdda.PREC_FP32: 5e-6}   # the MVP parity tolerances of the suite


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_no_alloc_mvp_matches_allocating_entry_point_twice():
    import torch
    nocc, L = 300, 4
    n, addr = bdda.aggregate(nocc, 1.0, 2.8, 17)
    rng = np.random.default_rng(17)
    x = rng.standard_normal((3 * nocc, L)) + 1j * rng.standard_normal((3 * nocc, L))
    diag = rng.standard_normal(3 * nocc) + 1j * rng.standard_normal(3 * nocc) + 4.0
    op = bdda.Operator(n, 0.02, 2 * np.pi / 0.55)
    op.set_dipoles(addr)
    for prec, dt in ((bdda.PREC_FP64, torch.complex128), (bdda.PREC_FP32, torch.complex64)):
        xd = torch.from_numpy(np.ascontiguousarray(x.T)).to(dt).cuda()
        dd = torch.from_numpy(diag).to(dt).cuda()
        jd = (1.0 / dd).contiguous()
        ref = torch.zeros_like(xd)
        torch.cuda.synchronize()
        op.mvp_device(xd.data_ptr(), ref.data_ptr(), L, 3 * nocc, 3 * nocc, prec=prec, diag=dd.data_ptr(),
                      jpre=jd.data_ptr())
        torch.cuda.synchronize()
        want = ref.cpu().numpy()
        for _call in range(2):
            out = torch.full_like(xd, float("nan"))
            torch.cuda.synchronize()
            op.mvp_device_noalloc(xd.data_ptr(), out.data_ptr(), L, 3 * nocc, 3 * nocc, prec=prec,
                                  diag=dd.data_ptr(), jpre=jd.data_ptr())
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            assert np.all(np.isfinite(got))
            assert _rel(got, want) <= TOL[prec]


def test_no_alloc_mvp_rejects_workspace_beyond_fixed_scratch():
    import torch
    nocc, L = 16384, 32
    n, addr = bdda.aggregate(nocc, 1.0, 2.8, 1)
    op = bdda.Operator(n, 0.02, 2 * np.pi / 0.55, prec=bdda.PREC_FP32)
    op.set_dipoles(addr)
    x = torch.zeros((L, 3 * nocc), dtype=torch.complex64, device="cuda")
    with pytest.raises(bdda.BddaError) as ei:
        op.mvp_device_noalloc(x.data_ptr(), x.data_ptr(), L, 3 * nocc, 3 * nocc, prec=bdda.PREC_FP32)
    assert ei.value.code == bdda.ERR_INVALID
    assert "scratch" in str(ei.value)


def test_no_alloc_mvp_allocates_nothing_and_needs_no_cleared_scratch():
    """A fresh operator's no-allocation MVPs leave the device's free memory as
    it was, and a scratch left full of NaN by a larger box's call does not
    reach the next call's result."""
    import torch
    nocc, L = 300, 4
    n, addr = bdda.aggregate(nocc, 1.0, 2.8, 23)
    rng = np.random.default_rng(23)
    x = rng.standard_normal((3 * nocc, L)) + 1j * rng.standard_normal((3 * nocc, L))
    k = 2 * np.pi / 0.55
    xd = torch.from_numpy(np.ascontiguousarray(x.T)).cuda()
    # an earlier operator on the same box loads the code that holds the scratch
    warm = bdda.Operator(n, 0.02, k)
    warm.set_dipoles(addr)
    tmp = torch.empty_like(xd)
    warm.mvp_device_noalloc(xd.data_ptr(), tmp.data_ptr(), L, 3 * nocc, 3 * nocc, prec=bdda.PREC_FP64)
    torch.cuda.synchronize()
    # a larger box with NaN input fills the scratch with NaN
    nb, ab = bdda.aggregate(2000, 1.0, 2.8, 5)
    big = bdda.Operator(nb, 0.02, k)
    big.set_dipoles(ab)
    xn = torch.full((2, 3 * ab.size), float("nan"), dtype=torch.complex128, device="cuda")
    yn = torch.empty_like(xn)
    big.mvp_device_noalloc(xn.data_ptr(), yn.data_ptr(), 2, 3 * ab.size, 3 * ab.size, prec=bdda.PREC_FP64)
    torch.cuda.synchronize()
    assert torch.isnan(yn).all()
    # a fresh operator: only no-allocation calls, and no change of free device memory
    fresh = bdda.Operator(n, 0.02, k)
    fresh.set_dipoles(addr)
    outs = [torch.empty_like(xd) for _ in range(2)]
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for out in outs:
        fresh.mvp_device_noalloc(xd.data_ptr(), out.data_ptr(), L, 3 * nocc, 3 * nocc, prec=bdda.PREC_FP64)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    # the allocating entry point on another operator of the same box is the reference
    ref = torch.empty_like(xd)
    warm.mvp_device(xd.data_ptr(), ref.data_ptr(), L, 3 * nocc, 3 * nocc, prec=bdda.PREC_FP64)
    torch.cuda.synchronize()
    want = ref.cpu().numpy()
    for out in outs:
        got = out.cpu().numpy()
        assert np.all(np.isfinite(got))
        assert _rel(got, want) <= TOL[bdda.PREC_FP64]
