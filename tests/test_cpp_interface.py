"""The C++ host interface (include/pdds.hpp) compiles against the C ABI with
the system C++ compiler and drives the library like a caller of the
reference's PDDSparseGM: layout on the host (CPU test), full estimate and
interface solve (GPU test)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "pdds_cpp_check.cpp")
OUT = os.path.join(ROOT, "pdds_gb300", "_build", "pdds_cpp_check")


@pytest.fixture(scope="module")
def exe():
    from pdds_gb300 import build as B
    lib = B.build()
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cuda_lib = "/usr/local/cuda/lib64"
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), SRC, "-o", OUT,
           lib, "-Wl,-rpath," + os.path.dirname(lib), "-L" + cuda_lib, "-Wl,-rpath," + cuda_lib, "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    assert "warning" not in res.stderr, res.stderr
    return OUT


def test_cpp_interface_host_layout(exe):
    import oracle as O
    res = subprocess.run([exe, "host"], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    parts = res.stdout.split()
    K, nnz, chk = int(parts[1]), int(parts[3]), float(parts[5])
    L = O.Layout((-1.0, -1.0), (1.0, 1.0), 4, 11)
    assert K == L.nknots
    x, y = np.zeros(K), np.zeros(K)
    x[L.work_idx], y[L.work_idx] = L.work_x, L.work_y
    want = 0.0
    for k in range(K):  # the same summation order as the C++ program
        want += x[k] * (k + 1) + y[k]
    assert abs(chk - want) <= 1e-12 * max(1.0, abs(want))
    assert nnz > 0


@pytest.mark.gpu
def test_cpp_interface_gpu_solve(exe):
    res = subprocess.run([exe, "gpu"], capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr
    line = res.stdout.strip().splitlines()[-1].split()
    rmse = float(line[1])
    assert rmse < 1e-2, res.stdout
    assert int(line[5]) > 0 and int(line[7]) > int(line[5])
