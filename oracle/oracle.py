"""ORACLE -- test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module; the product never does.  It is the checker, not the thing
measured.

Two oracles for larsjoost/wgls-rs-fft's batched power-of-two C2C FFT:

* ``ref_fft`` -- the reference's own single-precision Stockham radix-4/2 path,
  restated in C (``ref_stockham.c``: src/shaders.rs:8-106, src/lib.rs:517-579,
  661-669, 722-943).  Parity gate: max |a - b| <= 1e-3 per complex sample,
  the reference's VALIDATION_TOLERANCE (src/benchmark.rs:45, 272-297).
* ``fft64`` -- double precision with exactly reduced twiddles (``fft64.c``).
  Accuracy gate: relative L2 error <= 2e-6.

``ref_fft_numpy`` is an independent vectorised numpy restatement of the same
radix-4/2 stages used to cross-check the C restatement.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None
_lock = threading.Lock()

VALIDATION_TOLERANCE = 1e-3  # src/benchmark.rs:45
REL_L2_TOLERANCE = 2e-6


def build(force: bool = False) -> str:
    """Compile the C oracle with its Makefile into oracle/_build/."""
    if force or not os.path.exists(_LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(_LIB_PATH)
    return any(os.path.getmtime(os.path.join(_HERE, f)) > t
               for f in ("ref_stockham.c", "fft64.c", "Makefile"))


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            fp = ctypes.POINTER(ctypes.c_float)
            dp = ctypes.POINTER(ctypes.c_double)
            u32, u64, ci = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
            L.ref_fft_batch.argtypes = [fp, fp, u32, u32, ci]
            L.ref_fft_batch_mt.argtypes = [fp, fp, u32, u32, ci, ci]
            L.ref_twiddles.argtypes = [u32, fp]
            L.ref_prepare_input.argtypes = [fp, u64, ci, fp]
            L.ref_inverse_post.argtypes = [fp, u64, u32]
            L.fft64_batch_f32in.argtypes = [fp, dp, u64, u64, ci, ci]
            L.fft64_batch.argtypes = [dp, dp, u64, u64, ci, ci]
            L.fft64_dft.argtypes = [dp, dp, u64, ci]
            L.fft64_twiddle.argtypes = [u64, u64, dp, dp]
            for f in (L.ref_fft_batch, L.ref_fft_batch_mt, L.fft64_batch_f32in,
                      L.fft64_batch, L.fft64_dft):
                f.restype = ci
            _lib = L
        return _lib


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _as_c64(x):
    x = np.ascontiguousarray(x, dtype=np.complex64)
    if x.ndim == 1:
        x = x[None, :]
    return x


def ref_fft(x, inverse: bool = False, threads: int = 1) -> np.ndarray:
    """The reference's Stockham R4/R2 f32 path over a [batch, n] complex64 array."""
    x = _as_c64(x)
    b, n = x.shape
    out = np.empty_like(x)
    if b == 0:
        return out
    rc = lib().ref_fft_batch_mt(_fp(x.view(np.float32)), _fp(out.view(np.float32)),
                                n, b, int(inverse), int(threads))
    if rc != 0:
        raise ValueError("Transform length must be a non-zero power of two")
    return out


def fft64(x, inverse: bool = False, threads: int = 0) -> np.ndarray:
    """Double-precision FFT of a [batch, n] array; complex64 or complex128 input."""
    x = np.asarray(x)
    if x.ndim == 1:
        x = x[None, :]
    b, n = x.shape
    out = np.empty((b, n), dtype=np.complex128)
    if b == 0:
        return out
    thr = threads or min(os.cpu_count() or 1, 16)
    if x.dtype == np.complex64:
        x = np.ascontiguousarray(x)
        rc = lib().fft64_batch_f32in(_fp(x.view(np.float32)), _dp(out.view(np.float64)),
                                     n, b, int(inverse), thr)
    else:
        x = np.ascontiguousarray(x, dtype=np.complex128)
        rc = lib().fft64_batch(_dp(x.view(np.float64)), _dp(out.view(np.float64)),
                               n, b, int(inverse), thr)
    if rc != 0:
        raise ValueError("Transform length must be a non-zero power of two")
    return out


def dft64(x, inverse: bool = False) -> np.ndarray:
    """Direct O(N^2) double DFT of one row (pins fft64 for small N)."""
    x = np.ascontiguousarray(x, dtype=np.complex128).ravel()
    out = np.empty_like(x)
    rc = lib().fft64_dft(_dp(x.view(np.float64)), _dp(out.view(np.float64)), x.size, int(inverse))
    if rc != 0:
        raise ValueError("bad size")
    return out


def ref_twiddles(n: int) -> np.ndarray:
    t = np.empty(2 * n, dtype=np.float32)
    lib().ref_twiddles(n, _fp(t))
    return t.view(np.complex64)


def ref_prepare_input(x, inverse: bool) -> np.ndarray:
    """src/lib.rs:571-579 on a 1-D complex64 vector; returns the f32 interleave."""
    x = np.ascontiguousarray(x, dtype=np.complex64)
    out = np.empty(2 * x.size, dtype=np.float32)
    lib().ref_prepare_input(_fp(x.view(np.float32)), x.size, int(inverse), _fp(out))
    return out


def ref_inverse_post(x, n: int) -> np.ndarray:
    """src/lib.rs:661-669 (conjugate and scale by 1.0f/n) on a complex64 vector."""
    x = np.array(x, dtype=np.complex64, copy=True)
    lib().ref_inverse_post(_fp(x.view(np.float32)), x.size, n)
    return x


# ---------------------------------------------------------------------------
# numpy restatement of the same stages (independent of the C file)
# ---------------------------------------------------------------------------

def _cmul32(a, b):
    ar, ai = a.real.astype(np.float32), a.imag.astype(np.float32)
    br, bi = b.real.astype(np.float32), b.imag.astype(np.float32)
    re = ar * br - ai * bi
    im = ar * bi + ai * br
    return (re + 1j * im).astype(np.complex64)


def ref_fft_numpy(x, inverse: bool = False) -> np.ndarray:
    """Vectorised numpy restatement of src/shaders.rs R4/R2 + src/lib.rs driver."""
    x = _as_c64(x)
    b, n = x.shape
    if n == 0 or n & (n - 1):
        raise ValueError("Transform length must be a non-zero power of two")
    tw = ref_twiddles(n)  # same f32 twiddle rule, computed by the C file's libm
    data = np.conj(x) if inverse else x.copy()
    data = data.astype(np.complex64)
    log_n = n.bit_length() - 1
    p = 1
    for _ in range(log_n // 2):
        q = n >> 2
        tid = np.arange(q)
        k, j = tid % p, tid // p
        i0 = j * p + k
        xs = [data[:, i0 + m * q] for m in range(4)]
        t = k * (q // p)
        xs[1] = _cmul32(np.broadcast_to(tw[t], xs[1].shape), xs[1])
        xs[2] = _cmul32(np.broadcast_to(tw[2 * t], xs[2].shape), xs[2])
        xs[3] = _cmul32(np.broadcast_to(tw[3 * t], xs[3].shape), xs[3])
        s02, d02 = xs[0] + xs[2], xs[0] - xs[2]
        s13, d13 = xs[1] + xs[3], xs[1] - xs[3]
        out = np.empty_like(data)
        base = j * 4 * p + k
        out[:, base] = s02 + s13
        out[:, base + p] = (d02.real + d13.imag) + 1j * (d02.imag - d13.real)
        out[:, base + 2 * p] = s02 - s13
        out[:, base + 3 * p] = (d02.real - d13.imag) + 1j * (d02.imag + d13.real)
        data = out.astype(np.complex64)
        p *= 4
    if log_n % 2:
        h = n >> 1
        tid = np.arange(h)
        k, j = tid % p, tid // p
        i1 = j * p + k
        a, bb = data[:, i1], data[:, i1 + h]
        t = _cmul32(np.broadcast_to(tw[k * (h // p)], bb.shape), bb)
        out = np.empty_like(data)
        base = j * 2 * p + k
        out[:, base] = a + t
        out[:, base + p] = a - t
        data = out.astype(np.complex64)
    if inverse:
        scale = np.float32(1.0) / np.float32(n)
        data = (data.real * scale - 1j * (data.imag * scale)).astype(np.complex64)
    return data


# ---------------------------------------------------------------------------
# the reference's DSP pipeline stages (examples/parallel_pipeline.rs)
# ---------------------------------------------------------------------------

def _pcg_u32(v):
    v = v.astype(np.uint32)
    with np.errstate(over="ignore"):
        s = v * np.uint32(747796405) + np.uint32(2891336453)
        w = ((s >> ((s >> np.uint32(28)) + np.uint32(4))) ^ s) * np.uint32(277803737)
    return (w >> np.uint32(22)) ^ w


def ref_noise(batch: int, n: int, seed: int, sigma: float = 0.1) -> np.ndarray:
    """NOISE stage (examples/parallel_pipeline.rs:36-62): for sample tid of row
    batch_id, h1 = pcg(tid*1234567 + batch_id*7654321 + seed), h2 = pcg(h1 +
    999983), u1 = max(f32(h1) * 2.328306437e-10, 1e-7), u2 = f32(h2) *
    2.328306437e-10 * 6.283185307, r = sqrt(-2 ln u1) * sigma (0.1 there);
    returns the [batch, n] complex64 noise (r cos u2, r sin u2), computed in
    float32 like the shader."""
    tid = np.arange(n, dtype=np.uint64)[None, :]
    row = np.arange(batch, dtype=np.uint64)[:, None]
    with np.errstate(over="ignore"):
        v = ((tid * np.uint64(1234567) + row * np.uint64(7654321) + np.uint64(seed)) & np.uint64(0xFFFFFFFF))
    h1 = _pcg_u32(v.astype(np.uint32))
    with np.errstate(over="ignore"):
        h2 = _pcg_u32(h1 + np.uint32(999983))
    f = np.float32
    u1 = np.maximum(h1.astype(f) * f(2.328306437e-10), f(1e-7))
    u2 = h2.astype(f) * f(2.328306437e-10) * f(6.283185307)
    r = np.sqrt(f(-2.0) * np.log(u1)) * f(sigma)
    return (r * np.cos(u2) + 1j * (r * np.sin(u2))).astype(np.complex64)


def ref_pipeline(x, seed: int, sigma: float = 0.1) -> np.ndarray:
    """noise -> FFT -> Hann window over the bins -> IFFT (with 1/N) in FP64,
    the reference's six-stage pipeline without its DMA stages."""
    x = np.asarray(x)
    b, n = x.shape
    i = np.arange(n, dtype=np.float64)
    w = np.ones(n) if n == 1 else 0.5 * (1.0 - np.cos(2.0 * np.pi * i / (n - 1)))
    noisy = x.astype(np.complex128) + ref_noise(b, n, seed, sigma).astype(np.complex128)
    spec = fft64(noisy)
    return fft64(spec * w[None, :], inverse=True)


# ---------------------------------------------------------------------------
# metrics (src/benchmark.rs:272-297 and the relative-L2 gate)
# ---------------------------------------------------------------------------

def max_abs_err(a, b) -> float:
    """max over samples of |a - b| (complex norm), as src/benchmark.rs:285-289."""
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b)))


def rel_l2(a, ref) -> float:
    """||a - ref||_2 / ||ref||_2 over the whole batch."""
    a = np.asarray(a, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    den = np.linalg.norm(ref.ravel())
    num = np.linalg.norm((a - ref).ravel())
    return float(num / den) if den > 0 else float(num)
