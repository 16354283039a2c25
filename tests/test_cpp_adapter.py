"""The C++ adapter header (include/gpvmc_gb300.hpp) compiles and links
against the engine library (CPU), and a vmc.cpp-style driver written with it
reproduces the Python API's results on the GPU."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DRIVER = os.path.join(ROOT, "tests", "cpp", "vmc_driver.cpp")


def build_driver(tmp_path):
    from gpvmc_gb300 import build as b
    if not os.path.exists(b.LIB):
        b.build()
    exe = str(tmp_path / "vmc_driver")
    cuda_lib = "/usr/local/cuda/lib64"
    cmd = ["g++", "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), DRIVER, "-o", exe,
           "-L" + os.path.dirname(b.LIB), "-lgpvmc_gb300", "-L" + cuda_lib, "-lcudart",
           "-Wl,-rpath," + os.path.dirname(b.LIB) + ":" + cuda_lib]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_adapter_compiles_and_links(tmp_path):
    exe = build_driver(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.gpu
def test_driver_matches_python_api(tmp_path, engine):
    import math
    exe = build_driver(tmp_path)
    L, seed, W = 8, 1234, 4
    r = subprocess.run([exe, str(L), "0.25", "0.1", str(seed), str(W), "20", "10", "fp64"],
                       capture_output=True, text=True, check=True)
    tok = r.stdout.split()
    e_cpp = np.array([float(x) for x in tok[1:1 + W]])
    job = engine.Job(engine.StagFluxGroundState(L, 0.25 * math.pi, 0.1), walkers=W, seed=seed)
    job.set_measurements(3)
    job.init_walkers()
    job.walk(20 * L * L, 0)
    job.walk(10 * L * L, L * L)
    pj, n = job.projheis()
    np.testing.assert_allclose(e_cpp, pj[:, 0].real / n, rtol=0, atol=1e-14)
    assert int(tok[-1]) == 10
