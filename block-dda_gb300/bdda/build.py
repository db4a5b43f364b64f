"""Compile the CUDA library ``libbdda.so`` for sm_103a (in-tree, no cmake).

Each translation unit under ``block-dda_gb300/csrc`` is compiled in parallel
with ``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into
``block-dda_gb300/_lib/libbdda.so``.  Objects are rebuilt only when a source or
header is newer than the library.  Host code is compiled with
``-ffp-contract=off``: an aarch64 host compiler would otherwise fuse
multiply-adds that an x86-64 one keeps apart, and the seeded generators
(aggregates, directions) must give the same targets on both machines.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))   # block-dda_gb300/
REPO = os.path.dirname(PKG_ROOT)
CSRC = os.path.join(PKG_ROOT, "csrc")
LIBDIR = os.path.join(PKG_ROOT, "_lib")
LIB = os.path.join(LIBDIR, "libbdda.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _inputs():
    return _sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.hpp")) + \
        [os.path.join(REPO, "include", "bdda.h"), os.path.abspath(__file__)]


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(p) <= t for p in _inputs())


def _compile(nvcc, src, obj, verbose_ptxas):
    cmd = [nvcc, "-c", src, "-o", obj, "-O3", "-std=c++17", "-lineinfo", *ARCH,
           "-Xcompiler", "-fPIC", "-Xcompiler", "-O2", "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(REPO, "include"),
           "--expt-relaxed-constexpr"]
    if verbose_ptxas and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    return r.stderr


def build(force: bool = False, verbose_ptxas: bool = False, quiet: bool = True) -> str:
    """Build ``libbdda.so`` (if stale) and return its path."""
    if not force and up_to_date():
        return LIB
    nvcc = nvcc_path()
    objdir = os.path.join(LIBDIR, "obj")
    os.makedirs(objdir, exist_ok=True)
    srcs = _sources()
    objs = [os.path.join(objdir, os.path.basename(s) + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        futs = [ex.submit(_compile, nvcc, s, o, verbose_ptxas) for s, o in zip(srcs, objs)]
        logs = [f.result() for f in futs]
    if not quiet or verbose_ptxas:
        for s, log in zip(srcs, logs):
            if log.strip():
                print(f"--- {os.path.basename(s)}\n{log}", file=sys.stderr)
    tmp = LIB + ".tmp"
    cmd = [nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv, quiet=False))
