"""Host-side product code, no GPU: the C ABI library loads and exports every
declared symbol, the device FFT core (compiled for the CPU) matches numpy, and
the C++ target model (Mie polarizability, aggregates, incident fields, cross
sections) matches the reference's golden values and the oracle."""
import glob
import math
import os
import re

import numpy as np
import pytest

import bdda
from conftest import ROOT, golden
from oracle import physics


def _declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(bdda_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(lib):
    names = _declared_symbols()
    assert "bdda_op_create" in names and "bdda_solve" in names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(bdda.EXPORTS) <= names


def test_errors_are_reported_not_fatal(lib):
    import ctypes as ct
    h = ct.c_void_p()
    n = (ct.c_int * 3)(4, 4, 4)
    assert lib.bdda_op_create(ct.byref(h), n, 4, 1.0, 1.0, 0.0, 1) == bdda.ERR_INVALID
    assert b"f value" in lib.bdda_last_error()
    n = (ct.c_int * 3)(4, 601, 4)   # box sides up to 600: padded lines up to 1200 points
    assert lib.bdda_op_create(ct.byref(h), n, 3, 1.0, 1.0, 0.0, 1) == bdda.ERR_INVALID
    assert lib.bdda_op_set_graphs(None, 1) == bdda.ERR_INVALID
    assert b"null operator" in lib.bdda_last_error()


def _smooth(v):
    for p in (2, 3, 5):
        while v % p == 0:
            v //= p
    return v == 1


@pytest.mark.parametrize("N", [v for v in range(2, 1201) if _smooth(v)])
def test_device_fft_core_on_cpu(N):
    """Every 5-smooth length a box side up to 600 pads to (lengths past 512 run
    only the runtime-plan kernels)."""
    rng = np.random.default_rng(N)
    a = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    b = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    fa, rad = bdda.host_fft_line(a)
    assert int(np.prod(rad)) == N
    # forward output is a permutation of the DFT
    ref = np.fft.fft(a)
    assert np.allclose(np.sort_complex(np.round(fa, 8)), np.sort_complex(np.round(ref, 8)))
    # round trip and circular convolution, FP64 and FP32
    back, _ = bdda.host_fft_line(fa, inverse=True)
    assert np.max(np.abs(back / N - a)) < 1e-13
    fb, _ = bdda.host_fft_line(b)
    conv, _ = bdda.host_fft_line(fa * fb, inverse=True)
    cref = np.fft.ifft(np.fft.fft(a) * np.fft.fft(b))
    assert np.max(np.abs(conv / N - cref)) / np.max(np.abs(cref)) < 2e-15
    fa32, _ = bdda.host_fft_line(a, prec=2)
    fb32, _ = bdda.host_fft_line(b, prec=2)
    conv32, _ = bdda.host_fft_line(fa32 * fb32, inverse=True, prec=2)
    assert np.max(np.abs(conv32 / N - cref)) / np.max(np.abs(cref)) < 1e-6
    # double-float arithmetic (FP32 pairs): FP64-level accuracy
    fad, _ = bdda.host_fft_line(a, prec=3)
    fbd, _ = bdda.host_fft_line(b, prec=3)
    convd, _ = bdda.host_fft_line(fad * fbd, inverse=True, prec=3)
    assert np.max(np.abs(convd / N - cref)) / np.max(np.abs(cref)) < 1e-13
    # the z-axis schedule (composite register radices): same transform pair
    f16, r16 = bdda.host_fft_line(a, max_radix=16)
    g16, _ = bdda.host_fft_line(b, max_radix=16)
    c16, _ = bdda.host_fft_line(f16 * g16, inverse=True, max_radix=16)
    assert int(np.prod(r16)) == N and max(r16) <= 16
    assert np.allclose(np.sort_complex(np.round(f16, 8)), np.sort_complex(np.round(ref, 8)))
    assert np.max(np.abs(c16 / N - cref)) / np.max(np.abs(cref)) < 2e-15
    # the complex FP32 z schedule (first-stage radices up to 32): FP32 arithmetic, and FP64 as the
    # Green spectrum's transform runs it, in the same digit order
    f32s, r32 = bdda.host_fft_line(a, prec=2, max_radix=16)
    g32s, _ = bdda.host_fft_line(b, prec=2, max_radix=16)
    c32s, _ = bdda.host_fft_line(f32s * g32s, inverse=True, prec=2, max_radix=16)
    assert int(np.prod(r32)) == N and max(r32) <= 32 and all(r <= 16 for r in r32[1:])
    assert np.max(np.abs(c32s / N - cref)) / np.max(np.abs(cref)) < 1e-6
    for mr, f32, r32x in ((16, f32s, r32), (8, fa32, None)):   # z, then the x / y schedule
        f32d, r32d = bdda.host_fft_line(a, prec=1, max_radix=mr, c64_schedule=True)
        g32d, _ = bdda.host_fft_line(b, prec=1, max_radix=mr, c64_schedule=True)
        c32d, _ = bdda.host_fft_line(f32d * g32d, inverse=True, prec=1, max_radix=mr, c64_schedule=True)
        assert r32x is None or r32d == r32x
        assert np.max(np.abs(f32d - f32)) <= 1e-5 * np.max(np.abs(f32d))
        assert np.max(np.abs(c32d / N - cref)) / np.max(np.abs(cref)) < 2e-15
    # pruned input: only the first nv values are read (the rest are poisoned in the hook)
    nv = max(1, N // 2)
    ap = a.copy()
    ap[nv:] = 0.0
    fp, _ = bdda.host_fft_line(a, nvalid=nv)
    fz, _ = bdda.host_fft_line(ap)
    assert np.max(np.abs(fp - fz)) <= 1e-12 * np.max(np.abs(fz))


def test_mie_a1b1_matches_reference_gmie():
    cases = golden("mie_ref.json")
    worst = 0.0
    for c in cases:
        a1, b1 = bdda.mie_a1b1(c["wl0"], c["rp"], complex(*c["eper"]), complex(*c["mper"]))
        ra, rb = complex(*c["a1"]), complex(*c["b1"])
        worst = max(worst, abs(a1 - ra) / abs(ra), abs(b1 - rb) / abs(rb))
    assert worst < 1e-11, worst


def test_polarizability_of_result_dat_run():
    g = golden("result_dat_N512.json")
    t = golden("target_N512.json")
    k = 2 * math.pi / 0.3
    # r_p = cbrt(3 vol / 4 pi) of dipole 0 (Target.cpp:14-19); the files store vol = 4.18879 r_pp^3
    r_p = (3.0 * t["vol"][0] * g["scale_factor"] ** 3 / (4.0 * math.pi)) ** (1.0 / 3.0)
    alpha = bdda.polarizability(0.3, r_p, complex(*g["eper"]), k)
    ref = complex(*g["alpha0"])
    assert abs(alpha - ref) / abs(ref) < 1e-12


@pytest.mark.parametrize("nocc,seed", [(1, 1), (64, 2), (1024, 1), (5000, 7)])
def test_aggregate_is_connected_and_exact(nocc, seed):
    n, addr = bdda.aggregate(nocc, 1.0, 2.8, seed)
    assert addr.size == nocc and np.unique(addr).size == nocc
    assert addr.min() >= 0 and addr.max() < np.prod(n)
    n2, addr2 = bdda.aggregate(nocc, 1.0, 2.8, seed)
    assert n2 == n and np.array_equal(addr, addr2)          # seeded, deterministic
    # box is tight and the cluster is face-connected
    nx, ny, nz = n
    ix, iy, iz = addr // (ny * nz), (addr // nz) % ny, addr % nz
    assert ix.min() == 0 and iy.min() == 0 and iz.min() == 0
    assert ix.max() == nx - 1 and iy.max() == ny - 1 and iz.max() == nz - 1
    occ = set(addr.tolist())
    seen, stack = {int(addr[0])}, [int(addr[0])]
    while stack:
        a = stack.pop()
        x, y, z = a // (ny * nz), (a // nz) % ny, a % nz
        for dx, dy, dz in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
            X, Y, Z = x + dx, y + dy, z + dz
            if 0 <= X < nx and 0 <= Y < ny and 0 <= Z < nz:
                b = (X * ny + Y) * nz + Z
                if b in occ and b not in seen:
                    seen.add(b)
                    stack.append(b)
    assert len(seen) == nocc


def test_aggregate_fractal_dimension():
    # radius of gyration follows Rg = (N/kf)^(1/Df) within a loose band
    for df in (1.8, 2.8):
        n, addr = bdda.aggregate(4000, 1.0, df, 3)
        nx, ny, nz = n
        pts = np.stack([addr // (ny * nz), (addr // nz) % ny, addr % nz], 1).astype(float)
        rg = np.sqrt(((pts - pts.mean(0)) ** 2).sum(1).mean())
        target = (4000 / 1.0) ** (1 / df)
        assert 0.6 * target < rg < 1.6 * target, (df, rg, target)


def test_incident_fields_match_oracle():
    t = golden("target_N512.json")
    n, lf = tuple(t["n"]), t["lf"] * 0.03
    addr = np.array(t["address"])
    k = 2 * math.pi / 0.3
    u, e, _ = physics.reference_incident_waves(4)
    B = bdda.incident_fields(n, lf, addr, k, u, e)
    Bo = physics.incident_fields(physics.positions(n, lf, addr), k, e, u)
    assert np.max(np.abs(B - Bo)) < 1e-12


def test_cross_sections_match_oracle():
    rng = np.random.default_rng(9)
    E = rng.standard_normal((30, 3)) + 1j * rng.standard_normal((30, 3))
    P = rng.standard_normal((30, 3)) + 1j * rng.standard_normal((30, 3))
    a0 = 1e-4 + 3e-5j
    got = bdda.cross_sections(10.0, a0, E, P)
    ref = physics.cross_sections(10.0, E, P, a0)
    for g_, r_ in zip(got, ref):
        assert np.allclose(g_, r_, rtol=1e-13, atol=0)


def test_f6_incident_fields_and_cross_sections_match_oracle():
    t = golden("target_N16_coated.json")
    n, lf = tuple(t["n"]), t["lf"] * 0.02
    addr = np.array(t["address"])
    k = 2 * math.pi / 0.45
    u, e, h = physics.reference_incident_waves(5)
    B = bdda.incident_fields(n, lf, addr, k, u, e, h)
    Bo = physics.incident_fields(physics.positions(n, lf, addr), k, e, u, h)
    assert B.shape == (6 * addr.size, 5)
    assert np.max(np.abs(B - Bo)) < 1e-12
    rng = np.random.default_rng(4)
    P = rng.standard_normal(B.shape) + 1j * rng.standard_normal(B.shape)
    ae, ah = 1e-4 + 3e-5j, 2e-6 + 1e-6j
    got = bdda.cross_sections(k, ae, B, P, ah)
    ref = physics.cross_sections(k, B, P, ae, ah)
    for g_, r_ in zip(got, ref):
        assert np.allclose(g_, r_, rtol=1e-13, atol=0)


def test_f6_polarizabilities_match_reference_gmie():
    g = golden("result_f6_BC_rpp20nm.json")
    worst = 0.0
    for c in g["cases"][::5]:
        t = g["targets"][c["target"]]
        r_p = (3.0 * t["vol"][0] * g["scale_factor"] ** 3 / (4.0 * math.pi)) ** (1.0 / 3.0)
        k = 2 * math.pi / c["wl0"]
        ae, ah = bdda.polarizabilities(c["wl0"], r_p, complex(*c["eper"]), k)
        for got, ref in ((ae, complex(*c["alpha_e0"])), (ah, complex(*c["alpha_h0"]))):
            worst = max(worst, abs(got - ref) / abs(ref))
    assert worst < 1e-9, worst
    d = bdda.diag_a([2.0, 4.0j], [0.5, 1.0])
    assert np.allclose(d, [0.5] * 3 + [2.0] * 3 + [-0.25j] * 3 + [1.0] * 3)
