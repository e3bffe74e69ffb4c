"""CPU: the population of absent output pages that precedes GPU writes to
pageable host memory (wgls-rs-fft_gb300/csrc/host_pages.h), compiled for the
host and run on fresh anonymous mappings: fresh contiguous outputs and rows
become present, present ones are left alone, written contents are kept (in
place), adjacent small rows are populated as one run, and outputs under
128 KB are not examined."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "host_pages.cpp")
CSRC = os.path.join(ROOT, "wgls-rs-fft_gb300", "csrc")


def test_host_pages(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "host_pages")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-I", CSRC, SRC, "-o", exe], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True)
    lines = out.stdout.splitlines()
    assert out.returncode == 0 and len(lines) == 8 and all(l.startswith("ok ") for l in lines), out.stdout
