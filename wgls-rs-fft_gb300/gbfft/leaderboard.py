"""Rivalry leaderboard, as the reference prints it (larsjoost/wgls-rs-fft
examples/rivalry_leaderboard.rs), with the GB300 executor registered.

For each N in {256, 1024, 16384, 65536, 2^20} and the reference's batch rule
(choose_batch_size, examples/rivalry_leaderboard.rs:147-166, capped at
MAX_TOTAL_SAMPLES = 16 Mi samples, src/benchmark.rs:47), every rival's
host-vector ``fft`` -- the complete pipeline: host to device, transform,
device to host -- is run 3 times untimed and 10 times timed
(src/benchmark.rs:106-149), and reported in MSamples/s and GFLOPS
(5 N log2 N flops per transform).  Validation follows
src/benchmark.rs:155-190 and 272-297: one forward transform of the
deterministic input x_i = (0.001 t, 0.001 sin 2 pi t), t = i / N, compared
sample by sample with the baseline at the reference's 1e-3 tolerance.  The
reference's baseline is its own wgpu executor, which cannot run here; the
baseline is numpy's FFT in float64 of the same input.

Rivals:
  * GB300 FP32            -- gbfft.GpuFft, the reference's GpuFft interface
  * GB300 split FP16      -- the tensor-core split form (N >= 2^15)
  * cuFFT (torch.fft)     -- batched C2C over the whole batch in one call
    (the reference's cuFFT wrapper plans batch = 1 and loops,
    src/cufft_wrapper.rs:49-54)

Run:  python -m gbfft.leaderboard [--sizes 256 1024 ...]
"""
from __future__ import annotations

import argparse
import math
import time
from dataclasses import dataclass
from typing import Callable, List, Optional, Sequence

import numpy as np

from ._lib import PREC_TC_FP16, GbfftError, status_string
from .gpu_fft import FftExecutor, GpuFft

MAX_TOTAL_SAMPLES = 16 * 1024 * 1024  # src/benchmark.rs:47
VALIDATION_TOLERANCE = 1e-3           # src/benchmark.rs:45
WARMUP_ITERS = 3
BENCH_ITERS = 10
FFT_SIZES = (256, 1024, 16384, 65536, 1048576)


def choose_batch_size(n: int) -> int:
    """examples/rivalry_leaderboard.rs:147-166"""
    if n <= 1024:
        batch = 1024
    elif n <= 16384:
        batch = 256
    elif n <= 65536:
        batch = 64
    elif n <= 262_144:
        batch = 16
    else:
        batch = 1
    while n * batch > MAX_TOTAL_SAMPLES and batch > 1:
        batch //= 2
    return max(batch, 1)


def pipeline_input(n: int, batch: int) -> List[np.ndarray]:
    """The reference's deterministic benchmark input (src/benchmark.rs:112-122), in f32."""
    t = (np.arange(n, dtype=np.float32) / np.float32(n)).astype(np.float32)
    row = (t * np.float32(0.001)).astype(np.float32) + 1j * (np.sin(t * np.float32(2 * np.pi)).astype(np.float32)
                                                             * np.float32(0.001))
    row = row.astype(np.complex64)
    return [row.copy() for _ in range(batch)]


@dataclass
class Result:
    name: str
    batch: int
    msamples_per_sec: Optional[float]
    gflops: Optional[float]
    status: str


class TorchCuFft(FftExecutor):
    """cuFFT through torch.fft over the whole batch (one batched C2C plan)."""

    def __init__(self, device: int = 0):
        import torch
        self._torch = torch
        self._dev = torch.device("cuda", device)

    def name(self) -> str:
        return "cuFFT (torch.fft, batched)"

    def _run(self, inputs: Sequence[np.ndarray], inverse: bool) -> List[np.ndarray]:
        if len(inputs) == 0:
            return []
        torch = self._torch
        host = torch.from_numpy(np.ascontiguousarray(np.stack(inputs).astype(np.complex64)))
        d = host.to(self._dev, non_blocking=False)
        y = torch.fft.ifft(d, dim=1) if inverse else torch.fft.fft(d, dim=1)
        return list(y.cpu().numpy())

    def fft(self, inputs):
        return self._run(inputs, False)

    def ifft(self, inputs):
        return self._run(inputs, True)


class SplitFormGpuFft(GpuFft):
    """GpuFft with the tensor-core split form (FP16 hi + lo) selected
    (covers N >= 2^15; smaller sizes report UNSUPPORTED)."""

    def __init__(self, device: int = 0):
        super().__init__(device)
        self.context.set_precision(PREC_TC_FP16)

    def name(self) -> str:
        return "GB300 split FP16 (tcgen05)"


def default_rivals() -> List[FftExecutor]:
    rivals: List[FftExecutor] = [GpuFft(), SplitFormGpuFft()]
    try:
        import torch
        if torch.cuda.is_available():
            rivals.append(TorchCuFft())
    except ImportError:
        pass
    return rivals


def baseline_fft(inputs: Sequence[np.ndarray]) -> np.ndarray:
    return np.fft.fft(np.stack(inputs).astype(np.complex128), axis=1)


def validate(out: Sequence[np.ndarray], ref: np.ndarray) -> Optional[float]:
    """None when every sample is within the tolerance, else the max |a - b|
    (src/benchmark.rs:272-297)."""
    err = float(np.max(np.abs(np.stack(out).astype(np.complex128) - ref))) if len(out) else 0.0
    return None if err <= VALIDATION_TOLERANCE else err


def run_rival(rival: FftExecutor, n: int, batch: int,
              clock: Callable[[], float] = time.perf_counter) -> Result:
    inputs = pipeline_input(n, batch)
    try:
        for _ in range(WARMUP_ITERS):
            rival.fft(inputs)
        t0 = clock()
        for _ in range(BENCH_ITERS):
            rival.fft(inputs)
        dt = (clock() - t0) / BENCH_ITERS
        out = rival.fft(inputs)
    except GbfftError as e:  # e.g. the split form below its smallest size
        return Result(rival.name(), batch, None, None, status_string(e.status))
    samples = float(n * batch)
    err = validate(out, baseline_fft(inputs))
    status = "PASS" if err is None else f"FAIL({err:.2e})"
    return Result(rival.name(), batch, samples / dt / 1e6, 5.0 * samples * math.log2(n) / dt / 1e9, status)


def format_table(n: int, results: Sequence[Result]) -> str:
    """The reference's table (examples/rivalry_leaderboard.rs:111-141)."""
    lines = [f"\n--- N = {n} ---",
             f"{'Implementation':>32} | {'Batch':>8} | {'MSamples/s':>14} | {'GFLOPS':>10} | {'Status':>8}",
             "-" * 84]
    for r in results:
        if r.msamples_per_sec is None:
            lines.append(f"{r.name:>32} | {r.batch:>8} | {'ERROR':>14} | {'-':>10} | {r.status:>8}")
        else:
            lines.append(f"{r.name:>32} | {r.batch:>8} | {r.msamples_per_sec:>14.2f} | {r.gflops:>10.2f} | "
                         f"{r.status:>8}")
    return "\n".join(lines)


def main(argv: Optional[Sequence[str]] = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--sizes", type=int, nargs="*", default=list(FFT_SIZES))
    args = ap.parse_args(argv)
    print("\n=== GB300 FFT RIVALRY LEADERBOARD ===")
    print("Measuring complete GPU pipeline performance (host-to-device + GPU compute + device-to-host)")
    rivals = default_rivals()
    for n in args.sizes:
        batch = choose_batch_size(n)
        print(format_table(n, [run_rival(r, n, batch) for r in rivals]))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
