"""Every compile-time y plan of the complex FP32 strided passes (-m gpu).

For each padded y length a box can produce (Py = smallest 5-smooth >= 2 ny,
ny = 1..256) the FP32 block MVP must agree with the FP64 block MVP to the FP32
tolerance.  The y passes stage z-column pairs with 16-byte copies into rows
padded to a multiple of 4; the z extents 3..7 cover pairs whose second
column is padding (odd nz) and tiles of one to a few columns.
"""
import numpy as np
import pytest

import bdda

pytestmark = pytest.mark.gpu

TOL32 = 5e-6


def _smooth_at_least(v):
    while True:
        t = v
        for p in (2, 3, 5):
            while t % p == 0:
                t //= p
        if t == 1:
            return v
        v += 1


def test_every_y_plan_fp32_vs_fp64():
    import torch
    rng = np.random.default_rng(11)
    seen = {}
    for ny in range(1, 257):
        seen.setdefault(_smooth_at_least(2 * ny), ny)
    for i, (Py, ny) in enumerate(sorted(seen.items())):
        n = (2, ny, 3 + i % 5)  # z extents 3..7: z tiles of one to a few columns
        N = int(np.prod(n))
        nocc = max(1, (2 * N) // 3)
        addr = np.sort(rng.choice(N, size=nocc, replace=False)).astype(np.int32)
        L = 1 + i % 3
        x = rng.standard_normal((3 * nocc, L)) + 1j * rng.standard_normal((3 * nocc, L))
        op = bdda.Operator(n, 0.03, 2 * np.pi / 0.55)
        op.set_dipoles(addr)
        assert op.info()[0][1] == Py
        ys = []
        for prec, dt in ((bdda.PREC_FP64, torch.complex128), (bdda.PREC_FP32, torch.complex64)):
            xd = torch.from_numpy(np.ascontiguousarray(x.T)).to(dt).cuda()
            yd = torch.zeros_like(xd)
            torch.cuda.synchronize()
            op.mvp_device(xd.data_ptr(), yd.data_ptr(), L, 3 * nocc, 3 * nocc, prec=prec)
            torch.cuda.synchronize()
            ys.append(yd.cpu().numpy().T.astype(np.complex128))
        y64, y32 = ys
        if nocc == 1:
            assert np.max(np.abs(y32)) == 0.0
            continue
        rel = np.linalg.norm(y32 - y64) / np.linalg.norm(y64)
        assert rel < TOL32, (Py, ny, rel)
