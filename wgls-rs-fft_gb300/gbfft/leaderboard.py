"""Rivalry leaderboard, as the reference prints it (larsjoost/wgls-rs-fft
examples/rivalry_leaderboard.rs), with the GB300 executor registered.

For each N in {256, 1024, 16384, 65536, 2^20} and the reference's batch rule
(choose_batch_size, examples/rivalry_leaderboard.rs:159-177, capped at
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
  * GB300 split FP16      -- the tensor-core split form (N >= 16)
  * cuFFT (torch.fft)     -- batched C2C over the whole batch in one call
    (the reference's cuFFT wrapper plans batch = 1 and loops,
    src/cufft_wrapper.rs:49-54)

With --ncu, each size is followed by the device-side counters of the GB300
rivals: the rival's transform of the same batch is run once plainly, then
under Nsight Compute twice -- a launch list (device time only, one pass, every
kernel inside an NVTX range), then the DRAM bytes of the dominant kernel
alone (its first launch in the range) -- and each kernel's launches and time,
and the dominant kernel's DRAM traffic and achieved DRAM bandwidth, are
printed beside the algorithmic traffic (16 bytes per sample per pass, 1 pass
up to N = 2^14, 2 above).

Run:  python -m gbfft.leaderboard [--sizes 256 1024 ...] [--ncu]
"""
from __future__ import annotations

import argparse
import csv
import io
import math
import os
import subprocess
import sys
import tempfile
import time
from dataclasses import dataclass
from typing import Callable, List, Optional, Sequence

import numpy as np

from ._lib import PREC_FP32, PREC_TC_FP16, GbfftError, status_string
from .gpu_fft import FftExecutor, GpuFft

MAX_TOTAL_SAMPLES = 16 * 1024 * 1024  # src/benchmark.rs:47
VALIDATION_TOLERANCE = 1e-3           # src/benchmark.rs:45
WARMUP_ITERS = 3
BENCH_ITERS = 10
FFT_SIZES = (256, 1024, 16384, 65536, 1048576)


def choose_batch_size(n: int) -> int:
    """examples/rivalry_leaderboard.rs:159-177"""
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
    (covers N >= 16; smaller sizes report UNSUPPORTED)."""

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


# ---- device-side counters (Nsight Compute) ---------------------------------

NCU_METRICS = ("gpu__time_duration.sum", "dram__bytes_read.sum", "dram__bytes_write.sum")
NCU_TIME_METRICS = NCU_METRICS[:1]   # launch list: every kernel in the range
NCU_DRAM_METRICS = NCU_METRICS[1:]   # the dominant kernel only, one launch
NCU_RANGE = "gbfft_measure"


@dataclass
class KernelCounters:
    kernel: str
    launches: int
    seconds: float
    dram_bytes: float


def _number(text: str) -> float:
    return float(text.replace(",", "").strip() or "nan")


def parse_ncu_csv(text: str) -> List[KernelCounters]:
    """Per-kernel totals from `ncu --csv --print-units base` output (one row
    per launch and metric; lines before the CSV header are skipped)."""
    lines = text.splitlines()
    start = next((i for i, l in enumerate(lines) if l.startswith('"ID"')), None)
    if start is None:
        return []
    time_scale = {"ns": 1e-9, "nsecond": 1e-9, "us": 1e-6, "usecond": 1e-6, "ms": 1e-3, "msecond": 1e-3,
                  "s": 1.0, "second": 1.0}
    byte_scale = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
    per_launch = {}  # (launch ID, kernel) -> {metric: value in seconds or bytes}
    for row in csv.DictReader(io.StringIO("\n".join(lines[start:]))):
        metric, unit = row["Metric Name"], row.get("Metric Unit", "")
        if metric not in NCU_METRICS:
            continue
        value = _number(row["Metric Value"])
        value *= time_scale.get(unit, 1e-9) if metric == "gpu__time_duration.sum" else byte_scale.get(unit, 1.0)
        per_launch.setdefault((row["ID"], row["Kernel Name"]), {})[metric] = value
    out = {}
    for (_, name), rec in per_launch.items():
        # drop the parameter list: it starts after the template's closing '>'
        # (template arguments may hold parentheses themselves, e.g. "(int)-1")
        short = (name[:name.index(">(") + 1] if ">(" in name else name.split("(")[0]).replace("void ", "").strip()
        k = out.setdefault(short, KernelCounters(short, 0, 0.0, 0.0))
        k.launches += 1
        k.seconds += rec.get("gpu__time_duration.sum", 0.0)
        k.dram_bytes += rec.get("dram__bytes_read.sum", 0.0) + rec.get("dram__bytes_write.sum", 0.0)
    return sorted(out.values(), key=lambda k: -k.seconds)


def ncu_child(n: int, precision: int) -> int:
    """Body of the profiled process: one untimed transform of the size's
    batch, then one inside the NVTX range the capture is limited to."""
    rival = SplitFormGpuFft() if precision == PREC_TC_FP16 else GpuFft()
    inputs = pipeline_input(n, choose_batch_size(n))
    rival.fft(inputs)
    import torch
    torch.cuda.nvtx.range_push(NCU_RANGE)
    rival.fft(inputs)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    return 0


def _kernel_regex(short: str) -> str:
    """ncu -k filter on a kernel's function name without namespace or
    template arguments: 'gbfft::fft_rows_kernel<10, 11>' -> 'regex:fft_rows_kernel'."""
    import re
    base = short.split("<")[0].split("::")[-1].strip()
    return "regex:" + re.escape(base)


def ncu_counters(n: int, precision: int, ncu: str = "ncu", run=subprocess.run) -> List[KernelCounters]:
    """Run the size's transform plainly, then (only if that exited 0) under
    ncu: first a launch list with device time only (one pass per launch), then
    the DRAM read/write bytes of the dominant kernel alone, one launch
    (-k <its name> -c 1).  The dominant kernel's DRAM bytes are that launch's
    times its launch count; the other kernels carry no DRAM figure (nan)."""
    child = [sys.executable, "-m", "gbfft.leaderboard", "--ncu-child", str(n), "--precision", str(precision)]
    env = dict(os.environ)
    pkg_parent = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env["PYTHONPATH"] = pkg_parent + os.pathsep + env.get("PYTHONPATH", "")
    plain = run(child, env=env, capture_output=True, text=True)
    if plain.returncode != 0:
        raise RuntimeError(f"plain run failed ({plain.returncode}): {plain.stderr[-400:]}")
    with tempfile.TemporaryDirectory() as d:
        log = os.path.join(d, "launches.csv")
        cmd = [ncu, "--metrics", ",".join(NCU_TIME_METRICS), "--clock-control", "none", "--nvtx", "--nvtx-include",
               f"{NCU_RANGE}/", "--print-units", "base", "--csv", "--log-file", log, *child]
        r = run(cmd, env=env, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"ncu failed ({r.returncode}): {r.stderr[-400:]}")
        with open(log) as f:
            counters = parse_ncu_csv(f.read())
        if not counters:
            return counters
        for k in counters:
            k.dram_bytes = float("nan")
        top = counters[0]
        log2 = os.path.join(d, "dram.csv")
        cmd = [ncu, "--metrics", ",".join(NCU_DRAM_METRICS), "--clock-control", "none", "--nvtx", "--nvtx-include",
               f"{NCU_RANGE}/", "-k", _kernel_regex(top.kernel), "-c", "1", "--print-units", "base", "--csv",
               "--log-file", log2, *child]
        r = run(cmd, env=env, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"ncu failed ({r.returncode}): {r.stderr[-400:]}")
        with open(log2) as f:
            one = parse_ncu_csv(f.read())
        if one and one[0].launches:
            top.dram_bytes = one[0].dram_bytes / one[0].launches * top.launches
        return counters


def format_counters(n: int, batch: int, label: str, counters: Sequence[KernelCounters]) -> str:
    passes = 1 if n <= 1 << 14 else 2
    alg = 16.0 * n * batch * passes
    total_t = sum(k.seconds for k in counters)
    lines = [f"  ncu, {label}: {sum(k.launches for k in counters)} launch(es), {total_t * 1e6:.1f} us on the device; "
             f"algorithmic traffic {alg / 1e6:.1f} MB ({passes} pass(es) x 16 B/sample) = "
             f"{(alg / total_t / 1e9) if total_t > 0 else float('nan'):.0f} GB/s"]
    for k in counters:
        if math.isnan(k.dram_bytes):
            lines.append(f"    {k.kernel:<48} x{k.launches:<3} {k.seconds * 1e6:>10.1f} us")
            continue
        bw = k.dram_bytes / k.seconds / 1e9 if k.seconds > 0 else float("nan")
        lines.append(f"    {k.kernel:<48} x{k.launches:<3} {k.seconds * 1e6:>10.1f} us  DRAM {k.dram_bytes / 1e6:>9.1f} MB"
                     f"  {bw:>7.0f} GB/s")
    return "\n".join(lines)


def main(argv: Optional[Sequence[str]] = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--sizes", type=int, nargs="*", default=list(FFT_SIZES))
    ap.add_argument("--ncu", action="store_true", help="print Nsight Compute counters of the GB300 rivals")
    ap.add_argument("--ncu-path", default="ncu")
    ap.add_argument("--ncu-child", type=int, default=None, help=argparse.SUPPRESS)
    ap.add_argument("--precision", type=int, default=PREC_FP32, help=argparse.SUPPRESS)
    args = ap.parse_args(argv)
    if args.ncu_child is not None:
        return ncu_child(args.ncu_child, args.precision)
    print("\n=== GB300 FFT RIVALRY LEADERBOARD ===")
    print("Measuring complete GPU pipeline performance (host-to-device + GPU compute + device-to-host)")
    rivals = default_rivals()
    for n in args.sizes:
        batch = choose_batch_size(n)
        print(format_table(n, [run_rival(r, n, batch) for r in rivals]))
        if args.ncu:
            for prec, label in ((PREC_FP32, "GB300 FP32"), (PREC_TC_FP16, "GB300 split FP16")):
                if prec == PREC_TC_FP16 and n < 1 << 15:
                    continue
                print(format_counters(n, batch, label, ncu_counters(n, prec, args.ncu_path)))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
