"""Wavelength x target sweep (``bdda_sweep``) on the GPU (-m gpu).

* the recorded f=6 BiCGSTAB-Jacobi runs of DDA_result_BC_rpp20nm.dat for the
  N8..N64 targets at eleven wavelengths, reproduced through one sweep call
  (material table, polarizabilities, fields, solves and cross sections all in
  the library) with the same bars as the per-run test;
* warm-started refinement across a fine wavelength grid gives the cold-start
  cross sections with fewer Krylov iterations (no more for f=6, whose small
  test target converges in few BiCGSTAB steps either way).
"""
import math

import numpy as np
import pytest

import bdda
from conftest import golden
from oracle import physics

pytestmark = pytest.mark.gpu


def _bc_material(tmp_path):
    g = golden("materials_ref.json")
    p = tmp_path / "material_bc.dat"
    with open(p, "w") as fh:
        fh.write("##  BC\n")
        for w, e, m in g["tables"]["bc"]["rows"]:
            fh.write("%r  (%r,%r) (%r,%r)\n" % (w, e[0], e[1], m[0], m[1]))
    return bdda.Material.load(str(p), g["tables"]["bc"]["density"])


def test_sweep_reproduces_recorded_f6_runs(tmp_path):
    g = golden("result_f6_BC_rpp20nm.json")
    bc = _bc_material(tmp_path)
    s = g["scale_factor"]
    names = list(g["targets"])
    targets = []
    for nm in names:
        t = g["targets"][nm]
        targets.append((t["n"], t["lf"] * s, t["address"], np.array(t["vol"]) * s ** 3, None))
    wl = sorted({c["wl0"] for c in g["cases"]})
    u, e, h = physics.reference_incident_waves(4)
    opts = bdda.solve_opts("bicgstab", jacobi=True, tol=g["tol"], itermax=g["itermax"])
    cross, res = bdda.sweep(wl, targets, [bc], u, e, h, opts=opts)
    assert cross.shape == (len(wl), len(names), 4, 3)
    nstrict = 0
    for c in g["cases"]:
        w, t = wl.index(c["wl0"]), names.index(c["target"])
        r = res[w][t]
        assert r["status"] == 0 and r["mie_evaluations"] == 1
        assert abs(r["alpha_e0"] - complex(*c["alpha_e0"])) < 1e-9 * abs(complex(*c["alpha_e0"]))
        cext, cabs, csca = cross[w, t, :, 0], cross[w, t, :, 1], cross[w, t, :, 2]
        rec = c["recorded"]
        mac = (cabs * 1e-12 / rec["mass_particle"]).mean()
        assert abs(mac - rec["mean_MAC"]) / rec["mean_MAC"] < 1e-3
        if c["oracle_iterations"] <= 8 and rec["mean_SSA"] > 0.05:
            nstrict += 1
            assert r["iterations"] == c["oracle_iterations"]
            for got, key in ((csca.mean(), "mean_Csca"), (mac, "mean_MAC"), ((csca / cext).mean(), "mean_SSA")):
                assert abs(got - rec[key]) / abs(rec[key]) < 6e-6, (c["target"], c["wl0"], key)
    assert nstrict >= 15


@pytest.mark.parametrize("f", [3, 6])
def test_sweep_warm_start_matches_cold(f):
    nocc, L = 1500, 4
    n, addr = bdda.aggregate(nocc, 1.0, 2.8, 23)
    m_const = bdda.Material.constant((1.75 + 0.3j) ** 2, 1.0, 1.8)
    lf = 0.018
    vol = np.full(nocc, lf ** 3)
    wl = [0.500, 0.505, 0.510, 0.515, 0.520]
    u, e, h = physics.reference_incident_waves(L)
    opts = bdda.solve_opts("bicgstab" if f == 6 else "cocg_rq", jacobi=True, precision=bdda.SOLVE_MIXED,
                           true_tol=1e-8, itermax=2000)
    runs = {}
    for warm in (False, True):
        cross, res = bdda.sweep(wl, [(n, lf, addr, vol, None)], [m_const], u, e, h if f == 6 else None, opts=opts,
                                warm_start=warm)
        assert all(r[0]["status"] == 0 and r[0]["true_res_max"] <= 1e-8 for r in res)
        runs[warm] = (cross, sum(r[0]["iterations"] for r in res))
    cold, warm = runs[False], runs[True]
    assert np.max(np.abs(warm[0] - cold[0]) / np.abs(cold[0])) < 1e-6
    assert warm[1] <= cold[1] if f == 6 else warm[1] < cold[1], (warm[1], cold[1])


def test_warm_start_device_with_padded_leading_dimension():
    import torch
    nocc, L = 700, 3
    n, addr = bdda.aggregate(nocc, 1.0, 2.8, 5)
    wl0, m = 0.55, 1.6 + 0.1j
    k = 2 * math.pi / wl0
    lf = 0.5 / (abs(m) * k)
    alpha = bdda.polarizability(wl0, lf * (3 / (4 * math.pi)) ** (1 / 3), m * m, k)
    diag = bdda.diag_a(np.full(nocc, alpha))
    u, e, _h = physics.reference_incident_waves(L)
    B = bdda.incident_fields(n, lf, addr, k, u, e)
    op = bdda.Operator(n, lf, k)
    op.set_dipoles(addr)
    nr, ld = 3 * nocc, 3 * nocc + 5
    Bd = torch.from_numpy(np.ascontiguousarray(B.T)).cuda()
    Dd = torch.from_numpy(diag).cuda()
    Xd = torch.zeros((L, ld), dtype=torch.complex128, device="cuda")
    o = bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED, true_tol=1e-8, itermax=2000)
    st = bdda.solve_device(op, Dd.data_ptr(), Bd.data_ptr(), nr, Xd.data_ptr(), ld, L, o, allow_not_converged=False)
    assert st["true_res_max"] <= 1e-8 and st["iterations"] > 0
    X1 = Xd[:, :nr].clone()
    ow = bdda.solve_opts("cocg_rq", precision=bdda.SOLVE_MIXED, true_tol=1e-8, itermax=2000, warm_start=True)
    st2 = bdda.solve_device(op, Dd.data_ptr(), Bd.data_ptr(), nr, Xd.data_ptr(), ld, L, ow, allow_not_converged=False)
    assert st2["iterations"] == 0 and st2["true_res_max"] <= 1e-8      # already converged: one residual, no solve
    assert torch.equal(Xd[:, :nr], X1) and torch.all(Xd[:, nr:] == 0)
    with pytest.raises(bdda.BddaError):                                # warm start needs refinement
        bdda.solve_device(op, Dd.data_ptr(), Bd.data_ptr(), nr, Xd.data_ptr(), ld, L,
                          bdda.solve_opts("cocg_rq", warm_start=True))
