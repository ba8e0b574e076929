"""The bookkeeping of the packed ensemble's batched launches (block ->
instance search, launch-sequence merging and its mismatch errors),
compiled for the host with nvcc and run without a GPU."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "spd_gb300", "csrc")


def test_batch_recorder_and_block_offsets(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "host_batch_check")
    subprocess.run([nvcc, "-std=c++17", "-O1", "-I", CSRC, os.path.join(HERE, "host_batch_check.cu"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
