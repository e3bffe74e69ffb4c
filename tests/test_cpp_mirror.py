"""The C++ host mirror (include/gbfft.hpp): compiles everywhere (CPU), and
its restatement of the reference's tests passes on a GB300 (gpu)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "test_gpu_fft.cpp")


def _compile(out_dir, lib_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = os.path.join(out_dir, "test_gpu_fft")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe,
           "-L", os.path.dirname(lib_path), "-lgbfft", "-Wl,-rpath," + os.path.dirname(lib_path)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_mirror_compiles(tmp_path, lib_built):
    _compile(str(tmp_path), lib_built)


@pytest.mark.gpu
def test_cpp_mirror_reference_tests(tmp_path, lib_built):
    exe = _compile(str(tmp_path), lib_built)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK" in r.stdout
