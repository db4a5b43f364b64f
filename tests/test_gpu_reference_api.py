"""The reference-named C++ entry points (include/bdda_reference_api.hpp), compiled
with g++ against libbdda.so and called like Solver.cpp does, against the oracle.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

import bdda
from conftest import ROOT
from oracle import krylov, mbt

pytestmark = pytest.mark.gpu


def _compile(tmp_path):
    exe = str(tmp_path / "refdemo")
    lib = os.path.dirname(bdda.lib_path())
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
                    os.path.join(ROOT, "tests", "cpp", "reference_api_demo.cpp"), "-L", lib, "-lbdda",
                    f"-Wl,-rpath,{lib}", "-o", exe], check=True)
    return exe


def test_reference_named_entry_points(tmp_path):
    prob = bdda.make_problem(120, 1.8 + 0.4j, seed=9, n_dirs=2)
    n, nocc, L = prob.n, prob.nocc, prob.B.shape[1]
    rng = np.random.default_rng(0)
    ncub = 3 * int(np.prod(n))
    p_hat = rng.standard_normal(ncub) + 1j * rng.standard_normal(ncub)
    tol, itermax = 1e-8, 300
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as fh:
        fh.write(struct.pack("<5i", *n, nocc, L))
        fh.write(struct.pack("<4d", prob.lf, prob.k, 0.0, tol))
        fh.write(struct.pack("<i", itermax))
        fh.write(np.asarray(prob.address, dtype="<i4").tobytes())
        fh.write(prob.diag.astype("<c16").tobytes())
        fh.write(np.asfortranarray(prob.B).astype("<c16").tobytes(order="F"))
        fh.write(p_hat.astype("<c16").tobytes())
    out = tmp_path / "out.bin"
    subprocess.run([_compile(tmp_path), str(inp), str(out)], check=True)
    raw = open(out, "rb").read()
    off = 0

    def take(count):
        nonlocal off
        a = np.frombuffer(raw, dtype="<c16", count=count, offset=off)
        off += 16 * count
        return a

    q = take(ncub)
    X = take(3 * nocc * L).reshape((3 * nocc, L), order="F")
    Q = take(3 * nocc * L).reshape((3 * nocc, L), order="F")
    R = take(L * L).reshape((L, L), order="F")
    iters = struct.unpack_from("<i", raw, off)[0]
    # MBT_fft_mvp vs the literal restatement of the reference
    q_ref = mbt.mbt_fft_mvp(n, 3, mbt.mbt_fft_init(n, 3, prob.lf, prob.k), p_hat)
    assert np.linalg.norm(q - q_ref) / np.linalg.norm(q_ref) < 1e-12
    # bl_cocg_rq_jacobi_mvp_fft vs the oracle restatement
    gh, P = mbt.green_hat(n, 3, prob.lf, prob.k)
    Xo, hist = krylov.bl_cocg_rq(lambda S: mbt.block_mvp(n, 3, gh, P, prob.address, prob.diag, S), prob.B, tol,
                                 itermax, diag=prob.diag, jacobi=True)
    assert iters == len(hist)
    assert np.linalg.norm(X - Xo) / np.linalg.norm(Xo) < 1e-6
    Qo, Ro = krylov.qr_reduced(prob.B)
    assert np.max(np.abs(Q - Qo)) < 1e-12 and np.max(np.abs(R - Ro)) < 1e-12 * np.max(np.abs(Ro))
