"""Generate the committed golden fixtures under tests/golden/.

    python tests/golden/make_golden.py

Fixtures (numpy .npz, complex64 inputs):
  c1.npz        -- the N=1024 workload: 8 rows re/im iid uniform[-1, 1) (seed 1)
                   plus one row sin(0.1 i) + 0j; outputs of the reference's
                   Stockham R4/R2 path restated in C (forward and inverse) and of
                   the FP64 oracle (forward and inverse, complex128).
  ref_signals.npz -- the reference's own test signals (tests/gpu_fft_test.rs:8-15,
                   tests/test_utils.rs:21-48, src/lib.rs:212-214,
                   src/benchmark.rs:204-217) with their FP64 spectra.
  sweep.npz     -- N = 2^0 .. 2^12, 3 rows each, uniform seed 7: inputs, FP64
                   forward spectra and reference-path forward outputs.

The reference itself (Rust + wgpu) cannot run here, so these outputs come from
the oracle; tests/test_oracle.py pins the oracle against the reference's own
known-answer tests and re-derives every fixture bit-for-bit.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.join(REPO, "wgls-rs-fft_gb300"))

import oracle as O  # noqa: E402
from gbfft import signals  # noqa: E402


def c1_input() -> np.ndarray:
    x = signals.uniform_c64(8, 1024, seed=1)
    return np.concatenate([x, signals.sin_row(1024)[None, :]], axis=0)


def ref_signals():
    n = 1024
    i = np.arange(n, dtype=np.float32)
    # tests/gpu_fft_test.rs:8-15: re = (i*0.1).sin(), im = (i*0.07).cos() (f32 args)
    rustfft_sig = (np.sin((i * np.float32(0.1)).astype(np.float64)).astype(np.float32)
                   + 1j * np.cos((i * np.float32(0.07)).astype(np.float64)).astype(np.float32)).astype(np.complex64)
    # src/lib.rs:212-214: x_i = 0.1 i
    ramp = (i * np.float32(0.1)).astype(np.complex64)
    # tests/test_utils.rs:21-34 at N=2048: 0.7 sin(2 pi 10 t) + 0.3 sin(2 pi 50 t), t = i/N
    n2 = 2048
    t = np.arange(n2, dtype=np.float64) / n2
    tone = (0.7 * np.sin(2 * np.pi * 10 * t) + 0.3 * np.sin(2 * np.pi * 50 * t)).astype(np.float32).astype(np.complex64)
    hann = (tone * signals.hann_window(n2)).astype(np.complex64)
    # src/benchmark.rs:204-217: t = i/N, (0.001 t, 0.001 sin(2 pi t)), N=1024
    tb = np.arange(n, dtype=np.float64) / n
    bench = (0.001 * tb + 1j * 0.001 * np.sin(2 * np.pi * tb)).astype(np.complex64)
    impulse = np.zeros(256, dtype=np.complex64)
    impulse[0] = 1.0
    return dict(rustfft_sig=rustfft_sig, ramp=ramp, tone2048=tone, hann2048=hann, bench1024=bench,
                impulse256=impulse)


def main():
    O.build()
    x = c1_input()
    np.savez_compressed(
        os.path.join(HERE, "c1.npz"),
        x=x,
        ref_fwd=O.ref_fft(x, inverse=False),
        ref_inv=O.ref_fft(x, inverse=True),
        f64_fwd=O.fft64(x, inverse=False),
        f64_inv=O.fft64(x, inverse=True),
    )
    sig = ref_signals()
    out = {}
    for k, v in sig.items():
        out[k] = v
        out[k + "_f64"] = O.fft64(v[None, :])[0]
    np.savez_compressed(os.path.join(HERE, "ref_signals.npz"), **out)
    sw = {}
    for L in range(0, 13):
        n = 1 << L
        xs = signals.uniform_c64(3, n, seed=7)
        sw[f"x{L}"] = xs
        sw[f"f64_{L}"] = O.fft64(xs)
        sw[f"ref_{L}"] = O.ref_fft(xs)
    np.savez_compressed(os.path.join(HERE, "sweep.npz"), **sw)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
