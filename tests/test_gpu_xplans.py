"""Every compile-time x plan of the complex FP32 strided passes (-m gpu).

For each padded x length a box can produce (Px = smallest 5-smooth >= 2 nx,
nx = 1..256) the FP32 block MVP must agree with the FP64 block MVP to the FP32
tolerance.  The x passes move z-column pairs of the padded T1 rows with
16-byte copies; the z extents 3..10 cover pairs whose second column is
padding (odd nz), partial and full 8-column tiles.
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


def test_every_x_plan_fp32_vs_fp64():
    import torch
    rng = np.random.default_rng(12)
    seen = {}
    for nx in range(1, 257):
        seen.setdefault(_smooth_at_least(2 * nx), nx)
    for i, (Px, nx) in enumerate(sorted(seen.items())):
        n = (nx, 2, 3 + i % 8)  # z extents 3..10
        N = int(np.prod(n))
        nocc = max(1, (2 * N) // 3)
        addr = np.sort(rng.choice(N, size=nocc, replace=False)).astype(np.int32)
        L = 1 + i % 3
        x = rng.standard_normal((3 * nocc, L)) + 1j * rng.standard_normal((3 * nocc, L))
        op = bdda.Operator(n, 0.03, 2 * np.pi / 0.55)
        op.set_dipoles(addr)
        assert op.info()[0][0] == Px
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
        assert rel < TOL32, (Px, nx, rel)
