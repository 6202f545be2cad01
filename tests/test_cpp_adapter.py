"""The header-style C++ front end (include/bembel_gb300/H2MatrixGPU.hpp):
compiled with g++ as C++11 (the standard Bembel builds with) against the library and run (host-only checks on the CPU,
assembly + products + solve on a GPU)."""
import os
import shutil
import subprocess

import pytest

from conftest import SPHERE

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def adapter_exe(tmp_path_factory):
    from bembel_gb300 import _lib
    _lib.load()  # builds the library if needed
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("adapter") / "adapter_check")
    libdir = os.path.dirname(_lib.LIB_PATH)
    cmd = [cxx, "-std=c++11", "-O1", "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "adapter_check.cpp"),
           "-L", libdir, "-lbembel_gb300", "-Wl,-rpath," + libdir, "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_adapter_host(adapter_exe):
    r = subprocess.run([adapter_exe, SPHERE], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


@pytest.mark.gpu
def test_adapter_gpu(adapter_exe):
    r = subprocess.run([adapter_exe, SPHERE, "gpu"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr
