"""Python mirror of the reference's executor interface, over the C ABI.

Same names, argument meaning and error behaviour as larsjoost/wgls-rs-fft:
  trait FftExecutor { name, fft, ifft, as_any }      src/lib.rs:32-45
  GpuFft::new / fft / ifft / is_gpu_available / Default   src/lib.rs:285-489, 946-950
Inputs are a sequence of equal-length 1-D complex rows (the reference's
&[Vec<Complex<f32>>]); results are a list of complex64 rows.  Errors raise
GbfftError carrying the reference's messages; an empty batch returns [].
"""
from __future__ import annotations

from typing import List, Sequence

import numpy as np

from ._lib import FORWARD, INVERSE, Context, GbfftError, is_available


class FftExecutor:
    """src/lib.rs:32-45"""

    def name(self) -> str:
        raise NotImplementedError

    def fft(self, inputs: Sequence[np.ndarray]) -> List[np.ndarray]:
        raise NotImplementedError

    def ifft(self, inputs: Sequence[np.ndarray]) -> List[np.ndarray]:
        raise NotImplementedError

    def as_any(self):
        return self


class GpuFft(FftExecutor):
    """GB300 executor with the reference GpuFft's interface."""

    def __init__(self, device: int = 0):
        self._ctx = Context(device)

    @classmethod
    def new(cls, device: int = 0) -> "GpuFft":
        """src/lib.rs:285-330 (raises GbfftError when no GB300 is usable)."""
        return cls(device)

    @classmethod
    def default(cls) -> "GpuFft":
        """src/lib.rs:946-950: like new(), but a missing GPU is fatal."""
        try:
            return cls(0)
        except GbfftError as e:
            raise SystemExit(f"No GPU available for default GpuFft instance: {e}")

    @staticmethod
    def is_gpu_available() -> bool:
        """src/lib.rs:381-389"""
        return is_available()

    @property
    def context(self) -> Context:
        return self._ctx

    def name(self) -> str:
        return "GB300 (sm_103a Stockham radix-16)"

    def _run(self, inputs, direction):
        if len(inputs) == 0:  # src/lib.rs:522-524
            return []
        n = len(inputs[0])
        if n <= 2048 and all(len(r) == n for r in inputs):
            # many short rows: marshalling each row costs more than one extra
            # copy, so stack them (at C speed) into one contiguous batch for the
            # contiguous entry, which checks the length the same way
            out = self._ctx.c2c_host(np.stack(inputs).astype(np.complex64, copy=False), direction)
            return list(out)
        # unequal lengths: the row entry reports the reference's error, in its order
        return self._ctx.c2c_host_rows(inputs, direction)

    def fft(self, inputs):
        """src/lib.rs:433-438: forward, unscaled."""
        return self._run(inputs, FORWARD)

    def ifft(self, inputs):
        """src/lib.rs:483-488: inverse scaled by 1/N."""
        return self._run(inputs, INVERSE)

    def benchmark_gpu_only(self, n: int, batch: int, warmup: int = 3, iters: int = 50) -> float:
        """src/lib.rs:673-707: seconds per device-only transform."""
        return self._ctx.bench_device(n, batch, FORWARD, warmup, iters)
