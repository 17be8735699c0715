"""Builds the native parts of the package in-tree.

* ``dpgsolver_gb300/lib/libdpg_gb300.so``: host set-up (C11, gcc) + residual kernels (CUDA, nvcc for sm_103a)
  behind the C ABI of ``include/dpg_gb300.h``.
* ``oracle/_build/liboracle_dg.so``: the CPU oracle (test infrastructure; plain C).

Translation units are compiled in parallel; no cmake.  ``python -m dpgsolver_gb300._build`` runs it.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "dpgsolver_gb300")
OBJ = os.path.join(PKG, "_build")
LIB_DIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIB_DIR, "libdpg_gb300.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_LIB = os.path.join(ORACLE_DIR, "_build", "liboracle_dg.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build dpgsolver_gb300")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + proc.stdout)


def _newer(src: list[str], dst: str) -> bool:
    if not os.path.exists(dst):
        return True
    t = os.path.getmtime(dst)
    return any(os.path.getmtime(s) > t for s in src)


def build_library(force: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(PKG, "host"), "-I" + os.path.join(PKG, "csrc")]
    headers = glob.glob(os.path.join(ROOT, "include", "*.h")) + glob.glob(os.path.join(PKG, "host", "*.h")) \
        + glob.glob(os.path.join(PKG, "host", "*.inc")) + glob.glob(os.path.join(PKG, "csrc", "*.cuh"))
    c_src = sorted(glob.glob(os.path.join(PKG, "host", "*.c")))
    cu_src = sorted(glob.glob(os.path.join(PKG, "csrc", "*.cu")))
    nvcc = _nvcc()
    jobs = []
    objs = []
    for s in c_src:
        o = os.path.join(OBJ, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _newer([s] + headers, o):
            jobs.append(["gcc", "-O3", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-Wall", "-Wextra", *inc, "-c", s, "-o", o])
    for s in cu_src:
        o = os.path.join(OBJ, os.path.basename(s) + ".o")
        objs.append(o)
        if force or _newer([s] + headers, o):
            jobs.append([nvcc, "-O3", "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", *inc, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _newer(objs, LIB):
        _run([nvcc, "-shared", *ARCH, "-o", LIB, *objs, "-lm"])
    return LIB


def build_oracle(force: bool = False) -> str:
    """The CPU oracle (test infrastructure) is built by its own recipe, which never touches this package."""
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from oracle.oracle_py import build_oracle as _build_oracle

    return _build_oracle(force)


def build_all(force: bool = False) -> None:
    build_library(force)
    build_oracle(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
    print(ORACLE_LIB)
