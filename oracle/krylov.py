"""Oracle: block Krylov solvers of the reference, restated in numpy (complex128).

Test infrastructure only (see ``oracle/__init__.py``).  ``amul(S)`` is the block
operator ``S -> A S`` (diagonal included, see ``oracle.mbt.block_mvp``); the
Jacobi variants receive ``diag`` and form ``jpre = 1/diag`` themselves, exactly
as the reference does.  Every solver returns ``(X, history)`` where ``history``
is the list of the reference's per-iteration relative errors (the value the
reference prints), so tests can compare iteration counts.
"""
from __future__ import annotations

import numpy as np
import scipy.linalg as sla


def qr_reduced(a):
    """Thin QR by modified Gram-Schmidt with one re-orthogonalisation pass.

    Restates ``bl_krylov_mvp_fft/qr_reduced.cpp:9-31``: Hermitian inner products
    (``adjoint``, ``:21``), R(i,k) taken from the first pass only (``:18,22`` --
    ``tt`` starts at zero through the comma operator), R(k,k) = the real norm
    after the second pass (``:25-27``).
    """
    q = np.array(a, dtype=np.complex128, copy=True)
    n = q.shape[1]
    r = np.zeros((n, n), dtype=np.complex128)
    for k in range(n):
        tt = 0.0
        for _j in range(2):
            for i in range(k):
                s = np.vdot(q[:, i], q[:, k])
                if tt == 0.0:
                    r[i, k] = s
                q[:, k] = q[:, k] - s * q[:, i]
            tt = np.linalg.norm(q[:, k])
        r[k, k] = tt
        q[:, k] = q[:, k] / r[k, k]
    return q, r


def full_piv_solve(a, b):
    """Solve ``a x = b`` with complete pivoting (Eigen ``fullPivLu().solve``)."""
    a = np.array(a, dtype=np.complex128, copy=True)
    b = np.array(b, dtype=np.complex128, copy=True)
    n = a.shape[0]
    colperm = np.arange(n)
    for k in range(n):
        sub = np.abs(a[k:, k:])
        i, j = np.unravel_index(np.argmax(sub), sub.shape)
        i += k
        j += k
        if i != k:
            a[[k, i], :] = a[[i, k], :]
            b[[k, i], :] = b[[i, k], :]
        if j != k:
            a[:, [k, j]] = a[:, [j, k]]
            colperm[[k, j]] = colperm[[j, k]]
        if a[k, k] == 0:
            continue
        f = a[k + 1:, k] / a[k, k]
        a[k + 1:, k:] -= np.outer(f, a[k, k:])
        b[k + 1:, :] -= np.outer(f, b[k, :])
    y = np.zeros_like(b)
    for k in range(n - 1, -1, -1):
        if a[k, k] == 0:
            y[k] = 0
            continue
        y[k] = (b[k] - a[k, k + 1:] @ y[k + 1:]) / a[k, k]
    x = np.zeros_like(y)
    x[colperm] = y
    return x


def partial_piv_solve(a, b):
    """Solve ``a x = b`` with partial pivoting (Eigen ``partialPivLu().solve``)."""
    return sla.lu_solve(sla.lu_factor(a), b)


def _jacobi_setup(diag, B, jacobi):
    if not jacobi:
        return None, np.asarray(B, dtype=np.complex128)
    jpre = 1.0 / np.asarray(diag, dtype=np.complex128)
    return jpre, np.asarray(B, dtype=np.complex128) * jpre[:, None]


def bl_cocg_rq(amul, B, tol, itermax, diag=None, jacobi=False):
    """Block COCG-RQ (Gu et al. 2016).

    Non-Jacobi: ``bl_krylov_mvp_fft/bl_cocg_rq_mvp_fft.cpp:22-71`` (fullPivLu,
    ``:56,66``).  Jacobi: ``bl_cocg_rq_jacobi_mvp_fft.cpp:22-78`` (left scaling by
    ``jpre = 1/DIAG_A``, ``:22-27``; residual relative to ||B_pre|| ``:29,70``;
    partialPivLu ``:63,73``).  Unconjugated ``transpose`` for alpha/beta,
    Hermitian ``qr_reduced`` for the residual block.
    """
    jpre, Bp = _jacobi_setup(diag, B, jacobi)
    solve = partial_piv_solve if jacobi else full_piv_solve
    op = (lambda S: amul(S) * jpre[:, None]) if jacobi else amul
    bnorm = np.linalg.norm(Bp)
    X = np.zeros_like(Bp)
    Q, xi = qr_reduced(Bp)
    S = Q.copy()
    hist = []
    for _k in range(itermax):
        AS = op(S)
        alpha = solve(S.T @ AS, Q.T @ Q)
        X = X + S @ alpha @ xi
        Qn, tau = qr_reduced(Q - AS @ alpha)
        xi = tau @ xi
        err = np.linalg.norm(xi) / bnorm
        hist.append(err)
        if err < tol:
            break
        beta = solve(Q.T @ Q, tau.T @ Qn.T @ Qn)
        Q = Qn
        S = Q + S @ beta
    return X, hist


def bl_bicgstab(amul, B, tol, itermax, diag=None, jacobi=False):
    """Block BiCGSTAB (Tadano et al. 2009).

    ``bl_krylov_mvp_fft/bl_bicgstab_mvp_fft.cpp:21-98`` and the Jacobi variant
    ``bl_bicgstab_jacobi_mvp_fft.cpp:21-96``: one partial-pivot LU of
    ``R0til^H V`` reused for alpha and beta (``:58-59, :93``), zeta =
    tr(Z^H T)/tr(Z^H Z) (``:87``).
    """
    jpre, Bp = _jacobi_setup(diag, B, jacobi)
    op = (lambda S: amul(S) * jpre[:, None]) if jacobi else amul
    bnorm = np.linalg.norm(Bp)
    X = np.zeros_like(Bp)
    R = Bp.copy()
    P = R.copy()
    R0H = R.conj().T
    hist = []
    for _k in range(itermax):
        V = op(P)
        lu = sla.lu_factor(R0H @ V)
        alpha = sla.lu_solve(lu, R0H @ R)
        T = R - V @ alpha
        Z = op(T)
        qsi = np.trace(Z.conj().T @ T) / np.trace(Z.conj().T @ Z)
        X = X + P @ alpha + qsi * T
        R = T - qsi * Z
        err = np.linalg.norm(R) / bnorm
        hist.append(err)
        if err < tol:
            break
        beta = sla.lu_solve(lu, -R0H @ Z)
        P = R + (P - qsi * V) @ beta
    return X, hist


def bl_bicggr(amul, B, tol, itermax, diag=None, jacobi=False):
    """Block BiCGGR (Tadano et al. 2009).

    ``bl_krylov_mvp_fft/bl_bicggr_mvp_fft.cpp:18-116`` and
    ``bl_bicggr_jacobi_mvp_fft.cpp:18-117``: one initial MVP ``V = A R``
    (``:29-43``), two per iteration (``Y = A U`` ``:63-76``, ``W = A Rnew``
    ``:92-106``).
    """
    jpre, Bp = _jacobi_setup(diag, B, jacobi)
    op = (lambda S: amul(S) * jpre[:, None]) if jacobi else amul
    bnorm = np.linalg.norm(Bp)
    X = np.zeros_like(Bp)
    R = Bp.copy()
    P = R.copy()
    V = op(R)
    W = V.copy()
    R0H = R.conj().T
    hist = []
    for _k in range(itermax):
        alpha = partial_piv_solve(R0H @ V, R0H @ R)
        qsi = np.trace(W.conj().T @ R) / np.trace(W.conj().T @ W)
        S = P - qsi * V
        U = S @ alpha
        Y = op(U)
        X = X + qsi * R + U
        Rn = R - qsi * W - Y
        err = np.linalg.norm(Rn) / bnorm
        hist.append(err)
        if err < tol:
            break
        W = op(Rn)
        gamma = partial_piv_solve(R0H @ R, R0H @ Rn / qsi)
        R = Rn
        P = R + U @ gamma
        V = W + Y @ gamma
    return X, hist


SOLVERS = {"cocg_rq": bl_cocg_rq, "bicgstab": bl_bicgstab, "bicggr": bl_bicggr}


def true_residual(amul, B, X):
    """Per-column relative residual ||b_l - A x_l|| / ||b_l||."""
    R = B - amul(X)
    return np.linalg.norm(R, axis=0) / np.linalg.norm(B, axis=0)
