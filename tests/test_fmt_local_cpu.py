"""The per-node FMT math of the device path, checked on the host (no GPU).

tests/fmt_local_check.cu compiles the __host__ __device__ functions of
tramonto_gb300/csrc/tgpu_internal.h for the CPU and checks, for FMT1..FMT4 in
1, 2 and 3 dimensions at random weighted densities:
  * dPhi/dn against the oracle's FMT*_1stderiv restatements (1e-13 relative),
  * the reference-form second-derivative matrix against the oracle's
    d2phi_drb2_delta_rb / _theta_rb tables (1e-13 relative),
  * dPhi/dn against central differences of Phi, and the exact form against
    central differences of dPhi/dn (1e-5), and the exact form's symmetry.
"""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_fmt_local_math_matches_reference_tables(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "fmt_local_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", "-w", "-x", "cu", "-o", exe, os.path.join(HERE, "fmt_local_check.cu"),
                    "-I", os.path.join(ROOT, "oracle"), "-I", os.path.join(ROOT, "tramonto_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
