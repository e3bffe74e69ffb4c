"""Seeded synthetic signals for the benchmark workloads and the parity tests.

Counter-based generator built on the PCG hash of the reference's noise stage
(larsjoost/wgls-rs-fft examples/parallel_pipeline.rs:36-40):

    pcg(v):   s = v * 747796405 + 2891336453
              w = ((s >> ((s >> 28) + 4)) ^ s) * 277803737
              return (w >> 22) ^ w                      (all u32, wrapping)
    h(stream, seed, i) = pcg(pcg(seed ^ stream * 0x9E3779B9) + i)

Element i of a [batch, n] array is i = row * n + col (u32).  Real parts use
stream 0, imaginary parts stream 1.

    uniform[-1, 1):  ((h >> 8) * 2^-24) * 2 - 1          (exact in f32)
    normal N(0, 1):  Box-Muller in FP64 from u1 = ((h0 >> 8) + 1) 2^-24 in (0, 1]
                     and u2 = (h1 >> 8) 2^-24, rounded once to f32:
                     (r cos 2 pi u2, r sin 2 pi u2), r = sqrt(-2 ln u1)

numpy (host) and torch (device) versions produce identical integers; the
uniform path is bit-identical, the normal path may differ in the last f32 ulp
only where the host and device libm round a double differently.
"""
from __future__ import annotations

import numpy as np

_M32 = 0xFFFFFFFF
GOLDEN = 0x9E3779B9


def pcg_np(v: np.ndarray) -> np.ndarray:
    v = v.astype(np.uint32, copy=False)
    with np.errstate(over="ignore"):
        s = v * np.uint32(747796405) + np.uint32(2891336453)
        w = ((s >> ((s >> np.uint32(28)) + np.uint32(4))) ^ s) * np.uint32(277803737)
    return (w >> np.uint32(22)) ^ w


def stream_key(stream: int, seed: int) -> int:
    k = np.array([(seed ^ ((stream * GOLDEN) & _M32)) & _M32], dtype=np.uint32)
    return int(pcg_np(k)[0])


def hash_np(stream: int, seed: int, idx: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        return pcg_np(np.uint32(stream_key(stream, seed)) + idx.astype(np.uint32, copy=False))


def _chunks(total: int, chunk: int = 1 << 24):
    for a in range(0, total, chunk):
        yield a, min(total, a + chunk)


def uniform_c64(batch: int, n: int, seed: int) -> np.ndarray:
    """[batch, n] complex64, re/im iid uniform[-1, 1)."""
    total = batch * n
    out = np.empty(total, dtype=np.complex64)
    f = out.view(np.float32)
    for a, b in _chunks(total):
        idx = np.arange(a, b, dtype=np.uint64).astype(np.uint32)
        for st in (0, 1):
            h = hash_np(st, seed, idx)
            f[2 * a + st:2 * b:2] = ((h >> np.uint32(8)).astype(np.float32) * np.float32(2.0 ** -24)) * np.float32(2.0) - np.float32(1.0)
    return out.reshape(batch, n)


def normal_c64(batch: int, n: int, seed: int) -> np.ndarray:
    """[batch, n] complex64, re/im iid N(0, 1) (Box-Muller pair per sample)."""
    total = batch * n
    out = np.empty(total, dtype=np.complex64)
    f = out.view(np.float32)
    for a, b in _chunks(total):
        idx = np.arange(a, b, dtype=np.uint64).astype(np.uint32)
        h0 = hash_np(0, seed, idx)
        h1 = hash_np(1, seed, idx)
        u1 = ((h0 >> np.uint32(8)).astype(np.float64) + 1.0) * 2.0 ** -24
        u2 = (h1 >> np.uint32(8)).astype(np.float64) * 2.0 ** -24
        r = np.sqrt(-2.0 * np.log(u1))
        ang = 2.0 * np.pi * u2
        f[2 * a:2 * b:2] = (r * np.cos(ang)).astype(np.float32)
        f[2 * a + 1:2 * b:2] = (r * np.sin(ang)).astype(np.float32)
    return out.reshape(batch, n)


def sin_row(n: int) -> np.ndarray:
    """x_i = sin(0.1 i) + 0j with 0.1*i rounded in f32 first (the reference's
    test signal form (i as f32 * 0.1).sin(), tests/gpu_fft_test.rs:8-15)."""
    arg = np.arange(n, dtype=np.float32) * np.float32(0.1)
    return np.sin(arg.astype(np.float64)).astype(np.float32).astype(np.complex64)


def hann_window(n: int) -> np.ndarray:
    """w_i = 0.5 (1 - cos(2 pi i / (n - 1))) in FP64, rounded to f32
    (tests/test_utils.rs:39-48 computes the same formula in f32)."""
    if n == 1:
        return np.ones(1, dtype=np.float32)
    i = np.arange(n, dtype=np.float64)
    return (0.5 * (1.0 - np.cos(2.0 * np.pi * i / (n - 1)))).astype(np.float32)


# ---- device (torch) versions: same integers, generated in HBM ------------

def _pcg_torch(v):
    import torch
    m = 0xFFFFFFFF
    s = (v * 747796405 + 2891336453) & m
    w = ((torch.bitwise_right_shift(s, (s >> 28) + 4) ^ s) * 277803737) & m
    return ((w >> 22) ^ w) & m


def _hash_torch(stream, seed, idx):
    return _pcg_torch((idx + stream_key(stream, seed)) & 0xFFFFFFFF)


def normal_c64_torch(batch: int, n: int, seed: int, device="cuda"):
    """Device-side normal_c64 (complex64 tensor [batch, n])."""
    import torch
    total = batch * n
    out = torch.empty(total, 2, dtype=torch.float32, device=device)
    step = 1 << 24
    for a in range(0, total, step):
        b = min(total, a + step)
        idx = torch.arange(a, b, dtype=torch.int64, device=device)
        h0 = _hash_torch(0, seed, idx)
        h1 = _hash_torch(1, seed, idx)
        u1 = ((h0 >> 8).to(torch.float64) + 1.0) * 2.0 ** -24
        u2 = (h1 >> 8).to(torch.float64) * 2.0 ** -24
        r = torch.sqrt(-2.0 * torch.log(u1))
        ang = 2.0 * np.pi * u2
        out[a:b, 0] = (r * torch.cos(ang)).to(torch.float32)
        out[a:b, 1] = (r * torch.sin(ang)).to(torch.float32)
    return torch.view_as_complex(out).reshape(batch, n)


def uniform_c64_torch(batch: int, n: int, seed: int, device="cuda"):
    import torch
    total = batch * n
    out = torch.empty(total, 2, dtype=torch.float32, device=device)
    step = 1 << 24
    for a in range(0, total, step):
        b = min(total, a + step)
        idx = torch.arange(a, b, dtype=torch.int64, device=device)
        for st in (0, 1):
            h = _hash_torch(st, seed, idx)
            out[a:b, st] = ((h >> 8).to(torch.float32) * 2.0 ** -24) * 2.0 - 1.0
    return torch.view_as_complex(out).reshape(batch, n)


def _tone_params(batch: int, n: int, seed: int, tones: int):
    idx = np.arange(batch * tones, dtype=np.uint64).astype(np.uint32)
    bins = (hash_np(4, seed, idx) % np.uint32(n)).astype(np.int64).reshape(batch, tones)
    u_amp = (hash_np(5, seed, idx) >> np.uint32(8)).astype(np.float64) * 2.0 ** -24
    u_ph = (hash_np(6, seed, idx) >> np.uint32(8)).astype(np.float64) * 2.0 ** -24
    amp = (10.0 ** (6.0 * u_amp - 3.0)).reshape(batch, tones)      # log-uniform in [1e-3, 1e3]
    ph = (2.0 * np.pi * u_ph).reshape(batch, tones)                # uniform in [0, 2 pi)
    return bins, amp, ph


def tones_c64(batch: int, n: int, seed: int, tones: int = 64, sigma: float = 1e-2) -> np.ndarray:
    """[batch, n] complex64: per row `tones` complex exponentials at bins
    h(4, seed, .) mod n with amplitudes 10^U[-3,3] (h(5, .)) and phases
    U[0, 2 pi) (h(6, .)), built exactly in FP64 through the inverse DFT of
    their spectrum, plus complex N(0, sigma) noise (normal_c64 with seed + 1000;
    sigma is the standard deviation of each of re and im)."""
    bins, amp, ph = _tone_params(batch, n, seed, tones)
    spec = np.zeros((batch, n), dtype=np.complex128)
    rows = np.repeat(np.arange(batch), tones)
    np.add.at(spec, (rows, bins.ravel()), (n * amp * np.exp(1j * ph)).ravel())
    x = np.fft.ifft(spec, axis=1)
    x += sigma * normal_c64(batch, n, seed + 1000).astype(np.complex128)
    return x.astype(np.complex64)


def tones_c64_torch(batch: int, n: int, seed: int, ctx, tones: int = 64, sigma: float = 1e-2, device="cuda"):
    """Device-side tones_c64: the tone spectrum is scattered in HBM and turned
    into the time signal by this library's own FP32 inverse transform (which
    divides by n, hence the n factor), then the same noise is added."""
    import torch
    from ._lib import INVERSE, PREC_FP32
    bins, amp, ph = _tone_params(batch, n, seed, tones)
    spec = torch.zeros(batch * n, dtype=torch.complex128, device=device)
    flat = torch.from_numpy((np.arange(batch)[:, None] * n + bins).ravel()).to(device)
    vals = torch.from_numpy((n * amp * np.exp(1j * ph)).ravel()).to(device)
    spec.index_add_(0, flat, vals)
    spec = spec.to(torch.complex64).reshape(batch, n)
    x = torch.empty_like(spec)
    ctx.set_precision(PREC_FP32)
    ctx.c2c_device(spec, x, n, batch, INVERSE, stream=torch.cuda.current_stream().cuda_stream)
    x += sigma * normal_c64_torch(batch, n, seed + 1000, device=device)
    return x


def ragged_set(count: int = 10000, seed: int = 5, lo: int = 8, hi: int = 18):
    """The ragged workload: `count` transforms with log2 N uniform on
    {lo..hi} (h(2, seed, i) mod (hi-lo+1)), direction forward/inverse 50/50
    (bit 0 of h(3, seed, i)), packed back to back in descriptor order.
    Returns (descriptor array, total samples)."""
    from ._lib import FORWARD, INVERSE, RAGGED_DESC_DTYPE
    idx = np.arange(count, dtype=np.uint64).astype(np.uint32)
    logn = (lo + hash_np(2, seed, idx) % np.uint32(hi - lo + 1)).astype(np.uint32)
    dirs = np.where((hash_np(3, seed, idx) & np.uint32(1)) == 0, FORWARD, INVERSE).astype(np.int32)
    sizes = np.left_shift(np.uint64(1), logn.astype(np.uint64))
    offsets = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.uint64)
    d = np.empty(count, dtype=RAGGED_DESC_DTYPE)
    d["offset"], d["log2n"], d["direction"] = offsets, logn, dirs
    return d, int(sizes.sum())
