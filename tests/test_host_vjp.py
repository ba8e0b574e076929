"""The reverse-mode Jacobian-transpose products of the Euler maps used by
the adjoint kernels agree with dual-number (forward-mode) products of the
same device functions, compiled for the host with nvcc (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "spd_gb300", "csrc")


def test_reverse_mode_vjps_match_dual_numbers(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "host_vjp_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", "-x", "cu", "-I", CSRC, os.path.join(HERE, "host_vjp_check.cu"),
                    "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
