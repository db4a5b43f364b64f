"""Generate the committed golden fixtures under tests/golden/.

Run in a container where the nmoteki/block-DDA sources are mounted, with
``--ref PATH`` naming that source tree (required).  It reads the reference's own test
program, data files and recorded results as text, builds the reference's Mie
code with ``oracle/Makefile`` and writes small JSON fixtures.  The GPU machines
never run this; they only read the JSON it wrote.

Fixtures:
* ``mbt_f1_index_table.json`` -- the 27 ``n_ind`` patterns of the f=1
  known-answer leaf in ``module_tests/mvp_fft_tests/mvp_fft_example.cpp:37-103``.
* ``mie_ref.json`` -- a1, b1 from the reference's ``gmie_coeff`` and Q's from its
  ``gmie`` for a parameter sweep (polarizability pins).
* ``incident_dirs_ref.json`` -- propagation/polarisation vectors produced by
  libstdc++'s ``default_random_engine`` exactly as ``Incident_Wave.cpp:29-49``
  draws them (compiled and run here with g++).
* ``target_N512.json`` / ``target_N16_coated.json`` -- lattice addresses, volumes
  and material indices of ``DDA_target_0_agg_N512_kf1.0_Df2.8.out`` and
  ``DDA_target_2_agg_N16_kf1.0_Df2.8.out``.
* ``result_dat_N512.json`` -- the recorded cross sections of ``result.dat:14-42``
  (f=3 block COCG-RQ-Jacobi, tol 1e-2, N_inc 4) plus the oracle's per-iteration
  error history and solution-level cross sections for the same run.
* ``result_f6_BC_rpp20nm.json`` -- recorded f=6 (electric + magnetic dipoles)
  BiCGSTAB-Jacobi runs of ``DDA_result_BC_rpp20nm.dat`` for the N8..N64
  targets at eleven wavelengths, their target files, and the oracle's
  reproduction of each.
* ``target_N65536.npz`` -- the reference's largest aggregate,
  ``DDA_target_0_agg_N65536_kf1.0_Df2.8.out`` (box 137 x 135 x 176, 60,077
  monomer sites): box, lattice spacing, site volume and material, and the
  addresses in file order, delta-encoded (``address = cumsum(address_delta)``).
  The benchmark's ``--target-file`` workload reads it.  ``target_N1024.npz`` and
  ``target_N4096.npz`` hold the N1024 and N4096 aggregates the same way.
* ``materials_ref.json`` -- the four material tables and the eper the recorded
  runs used at each wavelength (interpolation pins).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import krylov, mbt, physics  # noqa: E402


def f1_table(ref):
    src = open(os.path.join(ref, "module_tests/mvp_fft_tests/mvp_fft_example.cpp")).read()
    pats = dict(re.findall(r"MatrixXi (n_ind_\d+_\d+)\(2,3\);\s*\1 << ([\d,]+);", src))
    vals = re.findall(r"if\(\(n_ind-(n_ind_\d+_\d+)\)\.norm\(\)==0\) MBT_elem <<(\d+);", src)
    table = []
    for name, v in vals:
        nums = [int(t) for t in pats[name].split(",")]
        table.append({"row0": nums[:3], "row1": nums[3:], "value": int(v)})
    assert len(table) == 27
    return table


def load_gmie(ref):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={ref}"], check=True)
    return ctypes.CDLL(os.path.join(ROOT, "oracle/_ref/libgmie_ref.so"))


def gmie_a1b1(lib, wl0, rp, ep, mp=1 + 0j, em=1 + 0j, mm=1 + 0j):
    a = (ctypes.c_double * 2)()
    b = (ctypes.c_double * 2)()
    args = [ctypes.c_double(v) for v in (wl0, rp, ep.real, ep.imag, mp.real, mp.imag, em.real, em.imag, mm.real, mm.imag)]
    lib.ref_gmie_a1b1(*args, a, b)
    return complex(a[0], a[1]), complex(b[0], b[1])


def gmie_q(lib, wl0, rp, ep, mp=1 + 0j, em=1 + 0j, mm=1 + 0j):
    o = (ctypes.c_double * 3)()
    args = [ctypes.c_double(v) for v in (wl0, rp, ep.real, ep.imag, mp.real, mp.imag, em.real, em.imag, mm.real, mm.imag)]
    lib.ref_gmie_q(*args, o)
    return o[0], o[1], o[2]


def mie_sweep(lib):
    cases = []
    for wl0 in (0.3, 0.55, 1.0):
        for m in (1.33 + 1e-8j, 1.78 + 0j, 1.95 + 0.79j, 2.3 + 0.6j, 1.7 + 0.5j):
            for rp in (0.005, 0.013, 0.03, 0.08):
                ep = m * m
                a1, b1 = gmie_a1b1(lib, wl0, rp, ep)
                qs, qa, qe = gmie_q(lib, wl0, rp, ep)
                cases.append({"wl0": wl0, "rp": rp, "eper": [ep.real, ep.imag], "mper": [1.0, 0.0],
                              "a1": [a1.real, a1.imag], "b1": [b1.real, b1.imag], "Q": [qs, qa, qe]})
    # BC at 0.3 um (material_bc.dat) and magnetic / coated cases
    for ep, mp in ((2.895 + 2.576j, 1 + 0j), (2.25 + 0j, 1 + 0j), (4.0 + 1.0j, 1.5 + 0.2j)):
        for rp in (0.02, 0.03, 0.04):
            a1, b1 = gmie_a1b1(lib, 0.3, rp, ep, mp)
            qs, qa, qe = gmie_q(lib, 0.3, rp, ep, mp)
            cases.append({"wl0": 0.3, "rp": rp, "eper": [ep.real, ep.imag], "mper": [mp.real, mp.imag],
                          "a1": [a1.real, a1.imag], "b1": [b1.real, b1.imag], "Q": [qs, qa, qe]})
    return cases


RNG_PROG = r"""
#include <cmath>
#include <cstdio>
#include <random>
int main(int argc, char** argv) {
  int L = atoi(argv[1]);
  std::default_random_engine re;
  std::uniform_real_distribution<double> urf{0, 1.0};
  for (int i = 1; i < L; ++i) {
    double a = urf(re), b = urf(re), c = urf(re);
    printf("%.17g %.17g %.17g\n", a, b, c);
  }
  return 0;
}
"""


def incident_dirs(n_inc=32):
    with tempfile.TemporaryDirectory() as td:
        src = os.path.join(td, "rng.cpp")
        exe = os.path.join(td, "rng")
        open(src, "w").write(RNG_PROG)
        subprocess.run(["g++", "-O0", "-o", exe, src], check=True)
        out = subprocess.run([exe, str(n_inc)], check=True, capture_output=True, text=True).stdout
    draws = [[float(t) for t in ln.split()] for ln in out.strip().splitlines()]
    u, e, h = physics.reference_incident_waves(n_inc)
    return {"n_inc": n_inc, "uniform_draws": draws, "uinc": u.tolist(),
            "einc_re": e.real.tolist(), "einc_im": e.imag.tolist()}


def target_fixture(ref, name, scale):
    n, lf, addr, vol, mat = physics.read_target_file(os.path.join(ref, name), 1.0)
    return {"source": name, "n": list(n), "lf": lf, "address": addr.tolist(),
            "vol": vol.tolist(), "material": mat.tolist(), "scale_factor_used_in_run": scale}


def target_npz(ref, name, path):
    n, lf, addr, vol, mat = physics.read_target_file(os.path.join(ref, name), 1.0)
    uv, um = np.unique(vol), np.unique(mat)
    if uv.size != 1 or um.size != 1:
        raise ValueError(f"{name}: expected one site volume and one material")
    delta = np.diff(addr.astype(np.int64), prepend=0).astype(np.int32)
    np.savez_compressed(path, source=np.array(name), n=np.array(n, dtype=np.int32), lf=np.float64(lf),
                        vol=np.float64(uv[0]), material=np.int32(um[0]), address_delta=delta)


def result_dat(ref, lib):
    txt = open(os.path.join(ref, "result.dat")).read()
    sec = txt[txt.index(SECTION):]
    recorded_text = sec[:sec.index("MAC_mie")] + sec[sec.index("MAC_mie"):].split("\n")[0] + "\n"
    rec = {}
    for key in ("mean_Csca", "std_Csca", "mean_MAC", "std_MAC", "mean_SSA", "std_SSA", "MAC_mie",
                "volume_particle", "num_element_occupy", "wl0", "N_inc"):
        m = re.search(rf"^{key}\t(\S+)", txt, re.M)
        rec[key] = float(m.group(1))
    # The run: r_pp = 30 nm (volume_particle = 476 * 4pi/3 * 0.03^3), BC eps at 0.3 um.
    scale = 0.03
    n, lf, addr, vol, _mat = physics.read_target_file(os.path.join(ref, "DDA_target_0_agg_N512_kf1.0_Df2.8.out"), scale)
    wl0 = 0.3
    k = 2 * math.pi / wl0
    eper = 2.895 + 2.576j
    rp = np.cbrt(vol * 3 / (4 * math.pi))
    alpha = np.array([3j * gmie_a1b1(lib, wl0, r, eper)[0] / (2 * k ** 3) for r in rp])
    diag = physics.diag_a(alpha)
    u, e, _h = physics.reference_incident_waves(4)
    B = physics.incident_fields(physics.positions(n, lf, addr), k, e, u)
    gh, P = mbt.green_hat(n, 3, lf, k)
    X, hist = krylov.bl_cocg_rq(lambda S: mbt.block_mvp(n, 3, gh, P, addr, diag, S), B, 1e-2, 300,
                                diag=diag, jacobi=True)
    cext, cabs, csca = physics.cross_sections(k, B, X, alpha[0])
    return {"recorded": rec, "recorded_text": recorded_text, "scale_factor": scale, "eper": [eper.real, eper.imag],
            "density": 1.8,
            "alpha0": [alpha[0].real, alpha[0].imag], "oracle_history": hist,
            "oracle_Cext": cext.tolist(), "oracle_Cabs": cabs.tolist(), "oracle_Csca": csca.tolist()}


SECTION = "####################### Start of result section #######################"


def _dat_sections(path, text=False):
    txt = open(path).read()
    secs = txt.split(SECTION)[1:]
    parsed = [dict(re.findall(r"^(\w+)\t(.*)$", sec, re.M)) for sec in secs]
    if text:
        for d, sec in zip(parsed, secs):
            d["_text"] = SECTION + sec.rstrip("\n") + "\n"
    return parsed


def result_f6(ref, lib):
    """Recorded f=6 runs of ``DDA_result_BC_rpp20nm.dat`` (BiCGSTAB-Jacobi, tol 1e-2,
    ``Solver.cpp:64-66``; BC particles of r_pp = 20 nm) for the targets
    ``DDA_target_0_agg_N{8,16,32,64}`` at all eleven wavelengths, with the
    oracle's reproduction of each (iteration count and mean cross sections)."""
    rows = _dat_sections(os.path.join(ref, "DDA_result_BC_rpp20nm.dat"), text=True)
    scale = 0.02
    names = [f"DDA_target_0_agg_N{N}_kf1.0_Df2.8.out" for N in (8, 16, 32, 64)]
    targets = {nm: target_fixture(ref, nm, scale) for nm in names}
    u, e, h = physics.reference_incident_waves(4)
    cases = []
    for r in rows:
        if r["target_fname"] not in targets:
            continue
        t = targets[r["target_fname"]]
        n, lf = tuple(t["n"]), t["lf"] * scale           # fixtures store the file's unscaled values
        addr = np.array(t["address"])
        vol = np.array(t["vol"]) * scale ** 3
        wl0 = float(r["wl0"])
        k = 2 * math.pi / wl0
        ep = complex(*[float(v) for v in r["eper_particle"].strip("()").split(",")])
        rp = np.cbrt(vol * 3 / (4 * math.pi))
        ab = [gmie_a1b1(lib, wl0, x, ep) for x in rp]
        ae = np.array([3j * a / (2 * k ** 3) for a, _b in ab])
        ah = np.array([3j * b / (2 * k ** 3) for _a, b in ab])
        diag = physics.diag_a(ae, ah)
        B = physics.incident_fields(physics.positions(n, lf, addr), k, e, u, h)
        gh, P = mbt.green_hat(n, 6, lf, k)
        X, hist = krylov.bl_bicgstab(lambda S: mbt.block_mvp(n, 6, gh, P, addr, diag, S), B, 1e-2, 300,
                                     diag=diag, jacobi=True)
        cext, cabs, csca = physics.cross_sections(k, B, X, ae[0], ah[0])
        mass = float(r["mass_particle"])
        rec = {key: float(r[key]) for key in ("mean_Csca", "std_Csca", "mean_MAC", "std_MAC", "mean_SSA", "std_SSA",
                                              "mass_particle", "volume_particle", "num_element_occupy", "wl0")}
        cases.append({"target": r["target_fname"], "wl0": wl0, "eper": [ep.real, ep.imag], "recorded": rec,
                      "alpha_e0": [ae[0].real, ae[0].imag], "alpha_h0": [ah[0].real, ah[0].imag],
                      "oracle_iterations": len(hist), "oracle_Cext": cext.tolist(), "oracle_Cabs": cabs.tolist(),
                      "recorded_text": r["_text"], "oracle_mean_Csca": float(csca.mean()),
                      "oracle_mean_MAC": float((cabs * 1e-12 / mass).mean()),
                      "oracle_mean_SSA": float((csca / cext).mean())})
    return {"scale_factor": scale, "tol": 1e-2, "itermax": 300, "solver": "bicgstab", "jacobi": True,
            "targets": targets, "cases": cases}


def materials_ref(ref):
    """The reference's material tables (``material_*.dat``, data files read as
    text) with the densities ``Material.cpp:31-57`` gives them, and the eper the
    recorded runs used at each wavelength (``DDA_result_BC_rpp20nm.dat``,
    ``DDA_result_MAGNETITE_rpp40nm.dat``): interpolation pins, e.g. magnetite
    at 0.3 um lies between the table rows 0.294118 and 0.303030."""
    dens = {"water": 1.0, "ice": 0.917, "bc": 1.8, "magnetite": 5.17}
    tables = {}
    for name in dens:
        rows = []
        for line in open(os.path.join(ref, f"material_{name}.dat")).read().splitlines():
            tok = line.split()
            if not tok or tok[0] == "##":
                continue
            e = [float(v) for v in tok[1].strip("()").split(",")]
            m = [float(v) for v in tok[2].strip("()").split(",")]
            rows.append([float(tok[0]), e, m])
        tables[name] = {"density": dens[name], "rows": rows}
    pins = {}
    for name, fn in (("bc", "DDA_result_BC_rpp20nm.dat"), ("magnetite", "DDA_result_MAGNETITE_rpp40nm.dat")):
        seen = {}
        for r in _dat_sections(os.path.join(ref, fn)):
            if "eper_particle" in r:  # homogeneous targets
                seen[float(r["wl0"])] = [float(v) for v in r["eper_particle"].strip("()").split(",")]
        pins[name] = sorted([w, e] for w, e in seen.items())
    return {"tables": tables, "recorded_eper": pins}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="nmoteki/block-DDA source tree")
    ap.add_argument("--only", nargs="*", help="write only these fixture files")
    args = ap.parse_args()
    ref = args.ref
    lib = load_gmie(ref)
    makers = {
        "mbt_f1_index_table.json": lambda: f1_table(ref),
        "mie_ref.json": lambda: mie_sweep(lib),
        "incident_dirs_ref.json": incident_dirs,
        "target_N512.json": lambda: target_fixture(ref, "DDA_target_0_agg_N512_kf1.0_Df2.8.out", 0.03),
        "target_N16_coated.json": lambda: target_fixture(ref, "DDA_target_2_agg_N16_kf1.0_Df2.8.out", 0.02),
        "result_dat_N512.json": lambda: result_dat(ref, lib),
        "result_f6_BC_rpp20nm.json": lambda: result_f6(ref, lib),
        "materials_ref.json": lambda: materials_ref(ref),
    }
    npz = {"target_N65536.npz": "DDA_target_0_agg_N65536_kf1.0_Df2.8.out",
           "target_N1024.npz": "DDA_target_0_agg_N1024_kf1.0_Df2.8.out",
           "target_N4096.npz": "DDA_target_0_agg_N4096_kf1.0_Df2.8.out"}
    for name, src in npz.items():
        if not args.only or name in args.only:
            target_npz(ref, src, os.path.join(HERE, name))
            print("wrote", name)
    out = {name: make() for name, make in makers.items() if not args.only or name in args.only}
    for name, obj in out.items():
        with open(os.path.join(HERE, name), "w") as fh:
            json.dump(obj, fh, indent=None, separators=(",", ":"))
        print("wrote", name)


if __name__ == "__main__":
    main()
