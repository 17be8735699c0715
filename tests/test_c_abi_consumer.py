"""The C ABI from plain C: tests/c_abi/consumer.c, compiled as C99 with warnings as errors against
include/dpg_gb300.h alone and linked to the built library, runs the host set-up, L2 error and restart round trip
(and, on a machine with a CUDA device, a residual and an RK step)."""
import os
import shutil
import subprocess

import pytest

import dpgsolver_gb300 as dg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(tmp_path, *extra):
    lib_dir = os.path.dirname(dg.LIB_PATH)
    exe = str(tmp_path / "consumer")
    cmd = ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_abi", "consumer.c"), "-L", lib_dir, "-ldpg_gb300",
           "-Wl,-rpath," + lib_dir, "-lm", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, str(tmp_path / "restart.msh"), *extra], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_c99_consumer(tmp_path):
    _run(tmp_path)


@pytest.mark.gpu
@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_c99_consumer_on_the_device(tmp_path):
    _run(tmp_path, "device")
