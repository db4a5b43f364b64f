"""Lattice spheres against Mie theory (-m gpu).

The reference's SPHERE target (``Target_manager.cpp:84-112``) is compared with
the Mie efficiencies of the volume-equivalent sphere, as its result files do
for every target (``Result_manager.cpp:137-175``, ``volume_equivalent_Mie_result``):
here the DDA side is the GPU solve (mixed precision, true residual 1e-8) and
the Mie side ``bdda_mie_q`` (pinned to the reference's gmie).

Two refractive indices (m = 1.33, non-absorbing; m = 1.95 + 0.79i) and two
lattice resolutions of the same sphere (|m| k d = 0.5 and 0.25; 12 and 24
dipoles across, 910-7144 dipoles).  Bounds, from the oracle solve of the same
targets: Qext within 5% at |m| k d = 0.5 and 2.5% at 0.25, Qabs within 7% and
3.5% (absorbing sphere), and the error at the finer lattice below half of the
coarse one.  One coarse case is also solved by the oracle (numpy block
COCG-RQ-Jacobi on the 3-D FFT operator): same Q's to 1e-6.
"""
import math

import numpy as np
import pytest

import bdda
from oracle import krylov, mbt, physics

pytestmark = pytest.mark.gpu

WL0 = 0.55
K = 2 * math.pi / WL0
BOUND = {0.5: {"qext": 0.05, "qabs": 0.07}, 0.25: {"qext": 0.025, "qabs": 0.035}}


def _sphere(m, nmax, diameter):
    n, lf, addr = bdda.shape_target("sphere", nmax, (diameter, diameter, diameter))
    nocc = addr.size
    a_eq = (3 * nocc * lf ** 3 / (4 * math.pi)) ** (1 / 3)
    alpha0 = bdda.polarizability(WL0, lf * (3 / (4 * math.pi)) ** (1 / 3), m * m, K)
    u = np.array([[0.0, 0.0, 1.0], [0.0, 0.0, 1.0]])
    e = np.array([[1, 0, 0], [0, 1, 0]], dtype=np.complex128)
    B = bdda.incident_fields(n, lf, addr, K, u, e)
    return n, lf, addr, a_eq, alpha0, B


def _q_dda(m, nmax, diameter, oracle=False):
    n, lf, addr, a_eq, alpha0, B = _sphere(m, nmax, diameter)
    diag = np.full(3 * addr.size, 1.0 / alpha0)
    if oracle:
        gh, P = mbt.green_hat(n, 3, lf, K)
        X, _ = krylov.bl_cocg_rq(lambda S: mbt.block_mvp(n, 3, gh, P, addr, diag, S), B, 1e-11, 1000,
                                 diag=diag, jacobi=True)
    else:
        op = bdda.Operator(n, lf, K)
        op.set_dipoles(addr)
        X, st = bdda.solve(op, diag, B, bdda.solve_opts("cocg_rq", jacobi=True, precision=bdda.SOLVE_MIXED,
                                                          true_tol=1e-8, itermax=2000), allow_not_converged=False)
        assert st["true_res_max"] <= 1e-8
    cext, cabs, _csca = bdda.cross_sections(K, alpha0, B, X)
    g = math.pi * a_eq ** 2
    return cext.mean() / g, cabs.mean() / g, a_eq


@pytest.mark.parametrize("m", [1.33 + 0j, 1.95 + 0.79j])
def test_lattice_sphere_converges_to_mie(m):
    d_coarse = 0.5 / (abs(m) * K)
    diameter = 12 * d_coarse
    errs = {}
    for mkd, nmax in ((0.5, 12), (0.25, 24)):
        qext, qabs, a_eq = _q_dda(m, nmax, diameter)
        _qsca, qabs_mie, qext_mie = bdda.mie_q(WL0, a_eq, m * m)
        e_ext = abs(qext / qext_mie - 1.0)
        assert e_ext <= BOUND[mkd]["qext"], (mkd, qext, qext_mie)
        errs[mkd] = [e_ext]
        if m.imag > 0:
            e_abs = abs(qabs / qabs_mie - 1.0)
            assert e_abs <= BOUND[mkd]["qabs"], (mkd, qabs, qabs_mie)
            errs[mkd].append(e_abs)
        else:
            assert abs(qabs) <= 1e-9 * qext  # no absorption without Im m
    for coarse, fine in zip(errs[0.5], errs[0.25]):
        assert fine < 0.5 * coarse, errs


def test_lattice_sphere_gpu_equals_oracle():
    m = 1.95 + 0.79j
    diameter = 12 * 0.5 / (abs(m) * K)
    qe, qa, _ = _q_dda(m, 12, diameter)
    qeo, qao, _ = _q_dda(m, 12, diameter, oracle=True)
    assert abs(qe - qeo) / qeo < 1e-6 and abs(qa - qao) / qao < 1e-6
