"""Double-float layer of the split path (df64.cuh, flux_df.cuh) against FP64 on the GPU.

tests/df64_check.cu is compiled for sm_103a and run: the conversion to FP64 must be bit-exact; reciprocal, square
root and product within 2^-44 relative (operands within 2^+-40); sums within 2^-45 of the larger operand; the
double-float Roe-Pike and Lax-Friedrichs fluxes (2D, 3D) within 3e-13 of the FP64 flux scale on random physical
states.
"""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_df64_layer_matches_fp64():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "df64_check")
    subprocess.run([nvcc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I" + os.path.join(ROOT, "dpgsolver_gb300", "csrc"), "-I" + os.path.join(ROOT, "include"),
                    "-o", exe, os.path.join(HERE, "df64_check.cu")], check=True)
    proc = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(proc.stdout)
    assert proc.returncode == 0, proc.stdout + proc.stderr
    assert "all checks passed" in proc.stdout
