"""The engine maps a uniform to a vertex in integers (device.cuh
scaled_floor), bit-identical to the reference's size_t(n * uniform())
including the double product's rounding.  CPU: compiled with nvcc as host
code and run over every lattice size on the path."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_scaled_floor_matches_double_product(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "check_scaled_floor")
    subprocess.run([nvcc, "-x", "cu", "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", os.path.join(ROOT, "gpvmc_gb300", "csrc"), "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "check_scaled_floor.cpp"), "-o", exe],
                   check=True, capture_output=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0" in r.stdout
