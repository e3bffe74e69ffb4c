"""CPU: the register butterflies of every FP32 kernel (Dft<2..32>, including the
radix-16 and radix-8 forms whose twiddles are applied up to a real factor that
the last additions take as FMAs) against a direct FP64 DFT, compiled for the
host by nvcc (no GPU needed).  Gate: relative L2 error <= 3e-7 (FP32 rounding)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "butterflies.cu")
CSRC = os.path.join(ROOT, "wgls-rs-fft_gb300", "csrc")


def test_butterflies_match_fp64_dft(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "butterflies")
    r = subprocess.run([nvcc, "-std=c++20", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
                        "-I", CSRC, SRC, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()
    errs = {int(out[i]): float(out[i + 1]) for i in range(0, len(out), 2)}
    assert sorted(errs) == [2, 4, 8, 16, 32]
    for radix, err in errs.items():
        assert err <= 3e-7, (radix, err)
