"""Oracle: targets, incident fields, DIAG_A and cross sections (numpy, FP64).

Test infrastructure only (see ``oracle/__init__.py``).
"""
from __future__ import annotations

import math

import numpy as np


# --------------------------------------------------------------------------
# libstdc++ default_random_engine + uniform_real_distribution<double>(0,1)
# --------------------------------------------------------------------------

class MinstdUniform:
    """``std::default_random_engine`` (minstd_rand0, seed 1) feeding
    ``uniform_real_distribution<double>{0,1}`` as libstdc++ implements it
    (``generate_canonical<double,53>``: two draws, sum/(r*r) with r = 2^31-2).

    Used by ``Incident_Wave::set_random_incident_directions``
    (``Incident_Wave.cpp:32-40``).
    """

    A = 16807
    M = 2147483647

    def __init__(self, seed: int = 1):
        self.state = seed % self.M or 1

    def _next(self) -> int:
        self.state = (self.A * self.state) % self.M
        return self.state

    def __call__(self) -> float:
        r = float(self.M - 1)          # max - min + 1 = 2147483646
        s = float(self._next() - 1)
        s = s + float(self._next() - 1) * r
        tmp = float(np.float64(r) * np.float64(r))
        ret = s / tmp
        if ret >= 1.0:
            ret = np.nextafter(1.0, 0.0)
        return ret


def angle_axis(psi: float, axis) -> np.ndarray:
    """Rotation matrix of ``Eigen::AngleAxisd(psi, axis)`` (Rodrigues)."""
    u = np.asarray(axis, dtype=np.float64)
    c, s = math.cos(psi), math.sin(psi)
    ux = np.array([[0.0, -u[2], u[1]], [u[2], 0.0, -u[0]], [-u[1], u[0], 0.0]])
    return c * np.eye(3) + (1.0 - c) * np.outer(u, u) + s * ux


def reference_incident_waves(n_inc: int, eper_m=1.0 + 0j, mper_m=1.0 + 0j):
    """Propagation, E and H polarisation vectors of ``Incident_Wave``.

    Default wave +z, x-polarised (``Incident_Wave.cpp:14-25``) followed by
    ``n_inc - 1`` random axis-angle rotations of it (``:29-49``).
    """
    u0 = np.array([0.0, 0.0, 1.0])
    e0 = np.array([1.0, 0.0, 0.0], dtype=np.complex128)
    h0 = np.array([0.0, np.sqrt(eper_m / mper_m), 0.0], dtype=np.complex128)
    us, es, hs = [u0], [e0], [h0]
    urf = MinstdUniform(1)
    for _i in range(1, n_inc):
        theta = math.acos(2.0 * urf() - 1.0)
        phi = 2 * math.pi * urf()
        nvec = np.array([math.sin(theta) * math.cos(phi), math.sin(theta) * math.sin(phi), math.cos(theta)])
        psi = 2 * math.pi * urf()
        rot = angle_axis(psi, nvec)
        us.append(rot @ u0)
        es.append(rot @ e0)
        hs.append(rot @ h0)
    return np.array(us), np.array(es), np.array(hs)


# --------------------------------------------------------------------------
# Mie coefficients of the volume-equivalent sphere (polarizability)
# --------------------------------------------------------------------------

def mie_a1b1(wl0, r_p, eper_p, mper_p=1.0 + 0j, eper_m=1.0 + 0j, mper_m=1.0 + 0j):
    """First Mie coefficients (a_1, b_1) as ``gmie/gmie_coeff.cpp:33-97`` computes
    them (BH83 eqs. 4.88 with the Kerker et al. 1983 permeability factors).

    D_n(y) by downward recurrence from 0 at nmx (``:43-46``); psi_n(x) from the
    downward ratio recurrence R_n = psi_n / psi_{n-1} started at x / (2 nmx + 1)
    with psi_0 = R_0 cos x (``:51-59``); chi_n(x) upward from chi_0 = -cos x,
    chi_1 = chi_0 / x - sin x (``:68-72``); xi = psi + i chi.
    """
    k0 = 2.0 * math.pi / wl0
    m_m = np.sqrt(complex(eper_m) * complex(mper_m))
    m_p = np.sqrt(complex(eper_p) * complex(mper_p))
    x = m_m * k0 * r_p
    m_r = m_p / m_m
    y = x * m_r
    nstop = int(math.floor(abs(x) + 4.0 * np.cbrt(abs(x)) + 2.0))
    nmx = max(nstop, int(math.ceil(abs(y)))) + 15
    dd = [0j] * nmx
    for n in range(nmx - 1, 1, -1):
        dd[n - 2] = n / y - 1.0 / (dd[n - 1] + n / y)
    rr = [0j] * (nmx + 1)
    rr[nmx] = x / (2.0 * nmx + 1.0)
    for n in range(nmx - 1, -1, -1):
        rr[n] = 1.0 / ((2.0 * n + 1.0) / x - rr[n + 1])
    psi0 = rr[0] * np.cos(x)
    psi1 = rr[1] * psi0
    chi0 = -np.cos(x)
    chi1 = (1.0 / x) * chi0 - np.sin(x)
    xi0, xi1 = psi0 + 1j * chi0, psi1 + 1j * chi1
    mp, mm = complex(mper_p), complex(mper_m)
    fa = mp / (mm * m_r) * dd[0] + 1.0 / x
    fb = mm * m_r / mp * dd[0] + 1.0 / x
    a1 = (fa * psi1 - psi0) / (fa * xi1 - xi0)
    b1 = (fb * psi1 - psi0) / (fb * xi1 - xi0)
    return complex(a1), complex(b1)


def polarizability(wl0, r_p, eper_p, k, mper_p=1.0 + 0j):
    """alpha_E = 3 i a_1 / (2 k^3) of a dipole of volume-equivalent radius r_p in
    vacuum (``Target_manager.cpp:232``)."""
    a1, _ = mie_a1b1(wl0, r_p, eper_p, mper_p)
    return 3j * a1 / (2.0 * k ** 3)


# --------------------------------------------------------------------------
# targets
# --------------------------------------------------------------------------

def read_target_file(path: str, scale_factor: float):
    """Parse a ``DDA_target_*.out`` file (``Target_manager.cpp:142-201``).

    Header: pp_radius, aggregate volume, coating volume, ``nx ny nz``, lf; then
    rows ``address vol material_index``.  lf and vol are scaled by
    scale_factor and scale_factor^3 (``:157,172``).
    """
    with open(path) as fh:
        lines = fh.read().splitlines()
    n = tuple(int(v) for v in lines[3].split())
    lf = float(lines[4]) * scale_factor
    rows = [ln.split() for ln in lines[5:] if ln.strip()]
    address = np.array([int(r[0]) for r in rows], dtype=np.int64)
    vol = np.array([float(r[1]) for r in rows]) * scale_factor ** 3
    mat = np.array([int(r[2]) for r in rows], dtype=np.int64)
    return n, lf, address, vol, mat


def positions(n, lf, address):
    """Physical coordinates (ix, iy, iz) * lf (``Target_manager.cpp:167-171``)."""
    nx, ny, nz = n
    address = np.asarray(address)
    ix = address // (ny * nz)
    iy = (address - ny * nz * ix) // nz
    iz = address - ny * nz * ix - nz * iy
    return np.stack([ix, iy, iz], axis=1).astype(np.float64) * lf


def incident_fields(pos, k, einc, uinc, hinc=None):
    """EHinc: f=3 rows ``einc_l exp(i k u_l . r_m)`` (``Target_manager.cpp:267-277``);
    with ``hinc`` (f=6) rows 6m..6m+5 hold ``[einc_l, hinc_l] exp(i k u_l . r_m)``
    (``Target_manager.cpp:280-291``)."""
    nocc = pos.shape[0]
    L = len(einc)
    f = 3 if hinc is None else 6
    out = np.zeros((f * nocc, L), dtype=np.complex128)
    for l in range(L):
        ph = np.exp(1j * k * (pos @ np.asarray(uinc[l])))
        amp = np.asarray(einc[l]) if hinc is None else np.concatenate([np.asarray(einc[l]), np.asarray(hinc[l])])
        out[:, l] = (ph[:, None] * amp[None, :]).reshape(-1)
    return out


def diag_a(alpha_e, alpha_h=None):
    """DIAG_A: 1/alpha_E over the 3 components (``Solver.cpp:33-36``); with
    ``alpha_h`` (f=6) 1/alpha_E then 1/alpha_H per dipole (``Solver.cpp:40-45``)."""
    ae = 1.0 / np.asarray(alpha_e, dtype=np.complex128)
    if alpha_h is None:
        return np.repeat(ae, 3)
    ah = 1.0 / np.asarray(alpha_h, dtype=np.complex128)
    return np.concatenate([np.repeat(ae[:, None], 3, 1), np.repeat(ah[:, None], 3, 1)], axis=1).reshape(-1)


def cross_sections(k: float, ehinc, pm, alpha0, alpha_h0=None):
    """Cext, Cabs, Csca per incident wave (``Result_manager.cpp:66-115``).

    Cext = 4 pi k Im(EH^H PM) over all rows.  f=3: Cabs = 4 pi k (Im(conj(1/alpha_0))
    - 2k^3/3) ||P||^2 with the polarizability of dipole 0 used for every dipole
    (``:73``).  f=6 (``alpha_h0`` given): the electric rows weigh with alpha_E(0),
    the magnetic rows with alpha_H(0) (``:94-99``).
    """
    cext = 4 * math.pi * k * np.imag(np.sum(np.conj(ehinc) * pm, axis=0))
    we = np.imag(np.conj(1.0 / alpha0)) - 2.0 * k ** 3 / 3.0
    if alpha_h0 is None:
        cabs = 4 * math.pi * k * we * np.sum(np.abs(pm) ** 2, axis=0)
    else:
        wh = np.imag(np.conj(1.0 / alpha_h0)) - 2.0 * k ** 3 / 3.0
        p6 = np.abs(pm.reshape(-1, 6, pm.shape[1])) ** 2
        cabs = 4 * math.pi * k * (we * p6[:, :3].sum(axis=(0, 1)) + wh * p6[:, 3:].sum(axis=(0, 1)))
    return cext, cabs, cext - cabs


# --------------------------------------------------------------------------
# materials and shape targets
# --------------------------------------------------------------------------

def material_eval(rows, wl0):
    """Linear interpolation of a material table in free-space wavelength,
    ``Material.cpp:88-124`` (same operation order): rows = [(wl0, eper, mper)]
    ascending; outside the table raises."""
    w = [r[0] for r in rows]
    if not (w[0] <= wl0 <= w[-1]):
        raise ValueError("wavelength outside the material table")
    for i in range(len(rows) - 1):
        if w[i] <= wl0 <= w[i + 1]:
            e0, e1 = complex(*rows[i][1]), complex(*rows[i + 1][1])
            m0, m1 = complex(*rows[i][2]), complex(*rows[i + 1][2])
            d = w[i + 1] - w[i]
            return e0 + (e1 - e0) / d * (wl0 - w[i]), m0 + (m1 - m0) / d * (wl0 - w[i])
    return complex(*rows[0][1]), complex(*rows[0][2])


def in_shape(shape, x, y, z, s):
    """``Target_manager::is_in_target_volume`` (``Target_manager.cpp:8-82``);
    shape 0 sphere, 1 cube, 2 ellipsoid, 3 cuboid, 4 cylinder, 5 rounded
    cylinder (whose second test ``r < z || z < l - r`` is always true above
    the lower cap, so the upper cap stays flat)."""
    if shape == 0:
        r = s[0] / 2.0
        return math.sqrt((x - r) ** 2 + (y - r) ** 2 + (z - r) ** 2) <= r
    if shape in (1, 3):
        return x <= s[0] and y <= s[1] and z <= s[2]
    if shape == 2:
        a, b, c = s[0] / 2.0, s[1] / 2.0, s[2] / 2.0
        return (x - a) * (x - a) / (a * a) + (y - b) * (y - b) / (b * b) + (z - c) * (z - c) / (c * c) <= 1.0
    r = s[0] / 2.0
    if shape == 4:
        return math.sqrt((x - r) ** 2 + (y - r) ** 2) <= r and z <= s[2]
    l = s[2]
    if z <= r:
        return math.sqrt((x - r) ** 2 + (y - r) ** 2 + (z - r) ** 2) <= r
    if r < z or z < l - r:
        return math.sqrt((x - r) ** 2 + (y - r) ** 2) <= r
    return math.sqrt((x - r) ** 2 + (y - r) ** 2 + (z - (l - r)) ** 2) <= r


def shape_target(shape, nmax, side_lengths):
    """``Target_manager::add_to_target_queue`` for a shape (``:84-112``):
    returns n, lf, occupied addresses."""
    mx = max(side_lengths)
    lf = mx / nmax
    n = [int(math.ceil(nmax * (s / mx))) for s in side_lengths]
    addr = []
    for ix in range(n[0]):
        for iy in range(n[1]):
            for iz in range(n[2]):
                if in_shape(shape, lf * ix, lf * iy, lf * iz, side_lengths):
                    addr.append(n[1] * n[2] * ix + n[2] * iy + iz)
    return tuple(n), lf, np.array(addr, dtype=np.int64)
