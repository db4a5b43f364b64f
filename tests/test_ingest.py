"""Target ingestion in the product library (no GPU): the target-file reader,
the shape generator, material tables and the per-dipole polarizabilities,
against the oracle's restatements and the reference's recorded values.

Files in the reference's formats are written into a temporary directory from
the committed fixtures (the target rows of ``DDA_target_2_agg_N16`` and the
four ``material_*.dat`` tables), so nothing here reads the reference tree.
"""
import math

import numpy as np
import pytest

import bdda
from conftest import golden
from oracle import physics


def _write_target(path, t, header=("1.0", "4.18879", "0.0")):
    with open(path, "w") as fh:
        fh.write("\n".join(header) + "\n")
        fh.write("%d %d %d\n" % tuple(t["n"]))
        fh.write("%r\n" % t["lf"])
        for a, v, m in zip(t["address"], t["vol"], t["material"]):
            fh.write("%d %r %d\n" % (a, v, m))


def _write_material(path, rows, name):
    with open(path, "w") as fh:
        fh.write("##  %s:\n##  wl0_um  (re(eper),im(eper)) (re(mper),im(mper))\n" % name)
        for w, e, m in rows:
            fh.write("%r  (%r,%r) (%r,%r)\n" % (w, e[0], e[1], m[0], m[1]))


def test_read_target_file(tmp_path):
    t = golden("target_N16_coated.json")
    p = tmp_path / "DDA_target_2_agg_N16.out"
    _write_target(p, t)
    n, lf, addr, vol, mat = bdda.read_target_file(str(p), 0.02)
    assert n == tuple(t["n"]) and abs(lf - t["lf"] * 0.02) < 1e-15
    assert np.array_equal(addr, t["address"]) and np.array_equal(mat, t["material"])
    assert np.allclose(vol, np.array(t["vol"]) * 0.02 ** 3, rtol=1e-15, atol=0)
    assert set(mat.tolist()) == {0, 1}                       # a coated target: two materials
    # the oracle's reader on the same file
    no, lfo, ao, vo, mo = physics.read_target_file(str(p), 0.02)
    assert no == n and lfo == lf and np.array_equal(ao, addr) and np.array_equal(vo, vol)


@pytest.mark.parametrize("bad", ["index", "address", "format", "header"])
def test_read_target_file_rejects_bad_files(tmp_path, bad):
    t = dict(golden("target_N16_coated.json"))
    p = tmp_path / "bad.out"
    if bad == "index":
        t["material"] = [2] + t["material"][1:]
    if bad == "address":
        t["address"] = [int(np.prod(t["n"]))] + t["address"][1:]
    _write_target(p, t, header=("1.0", "x", "0.0") if bad == "header" else ("1.0", "4.18879", "0.0"))
    if bad == "format":
        with open(p, "a") as fh:
            fh.write("12 0.5\n")
    with pytest.raises(bdda.BddaError):
        bdda.read_target_file(str(p), 1.0)


@pytest.mark.parametrize("shape", list(bdda.SHAPES))
@pytest.mark.parametrize("nmax,sides", [(8, (1.0, 1.0, 1.0)), (11, (0.6, 0.9, 1.5)), (16, (2.0, 2.0, 3.0))])
def test_shape_target_matches_oracle(shape, nmax, sides):
    n, lf, addr = bdda.shape_target(shape, nmax, sides)
    no, lfo, ao = physics.shape_target(bdda.SHAPES[shape], nmax, list(sides))
    assert n == no and lf == lfo and np.array_equal(addr, ao)
    assert addr.size > 0


def test_sphere_shape_volume():
    n, lf, addr = bdda.shape_target("sphere", 40, (1.0, 1.0, 1.0))
    v = addr.size * lf ** 3
    assert abs(v - math.pi / 6) / (math.pi / 6) < 0.03


def test_materials_interpolate_like_the_reference(tmp_path):
    g = golden("materials_ref.json")
    mats = {}
    for name, tab in g["tables"].items():
        p = tmp_path / f"material_{name}.dat"
        _write_material(p, tab["rows"], name)
        mats[name] = bdda.Material.load(str(p), tab["density"])
        assert mats[name].density == tab["density"]
    # the eper the recorded runs used (6 printed digits), incl. interpolated magnetite at 0.3 um
    for name, pins in g["recorded_eper"].items():
        for wl0, e in pins:
            got, mu = mats[name](wl0)
            assert abs(got - complex(*e)) / abs(complex(*e)) < 5e-6, (name, wl0)
            assert mu == 1.0
    # against the oracle at off-grid wavelengths
    rng = np.random.default_rng(3)
    for name, tab in g["tables"].items():
        w0, w1 = tab["rows"][0][0], tab["rows"][-1][0]
        for wl0 in np.concatenate([rng.uniform(w0, w1, 50), [w0, w1]]):
            e, m = mats[name](wl0)
            eo, mo = physics.material_eval(tab["rows"], wl0)
            assert e == eo and m == mo
        with pytest.raises(bdda.BddaError):
            mats[name](w1 * 1.01)
    c = bdda.Material.constant(2.0 + 0.5j, 1.0, 2.2)
    assert c(0.123) == (2.0 + 0.5j, 1.0 + 0j) and c.density == 2.2


def test_dipole_polarizabilities_cache_and_values(tmp_path):
    g = golden("materials_ref.json")
    t = golden("target_N16_coated.json")
    p = tmp_path / "bc.dat"
    _write_material(p, g["tables"]["bc"]["rows"], "bc")
    bc = bdda.Material.load(str(p), 1.8)
    coat = bdda.Material.constant(1.7 + 0.01j, 1.0, 1.0)
    vol = np.array(t["vol"]) * 0.02 ** 3
    wl0 = 0.55
    ae, ah, nev = bdda.dipole_polarizabilities(wl0, vol, [bc, coat], t["material"])
    assert nev == len(set(zip(vol.tolist(), t["material"])))
    k = 2 * math.pi / wl0
    for i in range(vol.size):
        r_p = np.cbrt(vol[i] * 3 / (4 * math.pi))
        mat = bc if t["material"][i] == 0 else coat
        e, _ = mat(wl0)
        a, b = bdda.polarizabilities(wl0, r_p, e, k)
        assert abs(ae[i] - a) <= 1e-12 * abs(a) and abs(ah[i] - b) <= 1e-12 * abs(b)  # b1 ~ r^5
    d = bdda.diag_a(ae, ah)
    assert np.allclose(d, physics.diag_a(ae, ah), rtol=1e-15, atol=0)
