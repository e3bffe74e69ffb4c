"""CPU: the shared-memory index maps of the single-pass tile and the global-pass
tile (fft_tiles.cuh) for every tile the kernels use -- single pass N = 2^4..2^14
with 16 samples a thread and 2^13 / 2^14 with 32; global passes of radix
2^5..2^10 with 16 samples a thread, 2^7..2^10 with 32, and the 8-column first
pass of radix 2^9 / 2^10 -- compiled for the host by nvcc from the kernels' own
index functions (no GPU needed).

Checked: every exchange and the first-pass output staging are bijections onto
the tile, read back where they were written (the staging as adjacent 16-byte
pairs for 8 columns), and each warp access takes the fewest shared-memory
wavefronts its width allows (2 for 8-byte lanes, 4 for 16-byte lanes),
including single-pass N = 2^5 / 2^6 / 2^7, where a warp spans 16 / 8 / 4
transforms and each transform's buffer is padded by one sample a thread so
that the buffers start on different banks."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT

SRC = os.path.join(ROOT, "tests", "cpp", "tile_maps.cu")
CSRC = os.path.join(ROOT, "wgls-rs-fft_gb300", "csrc")


def test_pass_tile_index_maps(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "tile_maps")
    r = subprocess.run([nvcc, "-std=c++20", "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include"),
                        "-I", CSRC, SRC, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.splitlines()
    single = [tuple(int(v) for v in line.split()[1:]) for line in out if line.startswith("rows ")]
    passes = [tuple(int(v) for v in line.split()[1:]) for line in out if line.startswith("pass ")]
    assert len(single) == 13 and len(passes) == 14
    small = {4: 0}  # no exchange at 2^4
    for logn, le, ok, w in single:
        assert ok == 1, (logn, le)
        assert w == small.get(logn, 2), ("single-pass exchange wavefronts", logn, le, w)
    for logr, le, cl, ok, wx, ws, wp in passes:
        assert ok == 1, (logr, le, cl)
        assert wx == 2, ("exchange wavefronts", logr, le, cl, wx)
        assert ws == 2, ("staging wavefronts", logr, le, cl, ws)
        assert wp == (4 if cl == 3 else 2), ("staging read-back wavefronts", logr, le, cl, wp)
