"""ctypes binding of the C ABI in include/gbfft.h.

There is no fallback: if libgbfft.so is missing or cannot be loaded, every
entry point raises.  The library is the only implementation of the transform.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from .build import LIB_PATH

FORWARD = -1
INVERSE = +1
PREC_FP32 = 0
PREC_TC_FP16 = 1
PREC_TC_BF16X3 = 2
PREC_TC_TF32 = 3
PREC_TC_BF16X6 = 4
WINDOW_NONE = 0
WINDOW_HANN = 1

OK = 0
ERR_INVALID_SIZE = 1
ERR_LENGTH_MISMATCH = 2
ERR_INVALID_ARGUMENT = 3
ERR_NO_DEVICE = 4
ERR_OUT_OF_MEMORY = 5
ERR_CUDA = 6
ERR_TIMEOUT = 7
ERR_UNSUPPORTED = 8

# Every symbol include/gbfft.h declares, with (restype, argtypes).
_vp = ctypes.c_void_p
_u64 = ctypes.c_uint64
_int = ctypes.c_int
_fp = ctypes.POINTER(ctypes.c_float)
SIGNATURES = {
    "gbfft_is_available": (_int, []),
    "gbfft_create": (_int, [_int, ctypes.POINTER(_vp)]),
    "gbfft_destroy": (None, [_vp]),
    "gbfft_last_error": (ctypes.c_char_p, [_vp]),
    "gbfft_status_string": (ctypes.c_char_p, [_int]),
    "gbfft_c2c_host": (_int, [_vp, _vp, _vp, _u64, _u64, _int]),
    "gbfft_c2c_host_rows": (_int, [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_u64), ctypes.POINTER(_vp), _u64, _int]),
    "gbfft_c2c_device": (_int, [_vp, _vp, _vp, _u64, _u64, _int, _vp]),
    "gbfft_c2c_device_noalloc": (_int, [_vp, _vp, _u64, _u64, _int, _vp]),
    "gbfft_ragged_plan_create": (_int, [_vp, _vp, ctypes.c_uint32, ctypes.POINTER(_vp)]),
    "gbfft_ragged_plan_set": (_int, [_vp, _int, _u64]),
    "gbfft_ragged_execute": (_int, [_vp, _vp, _vp, _u64, _int, _vp]),
    "gbfft_ragged_wait": (_int, [_vp, _vp]),
    "gbfft_ragged_launch_count": (_u64, [_vp]),
    "gbfft_ragged_plan_destroy": (None, [_vp]),
    "gbfft_ragged_device": (_int, [_vp, _vp, _vp, _u64, _vp, ctypes.c_uint32, _vp]),
    "gbfft_bench_device": (_int, [_vp, _u64, _u64, _int, _int, _int, ctypes.POINTER(ctypes.c_double)]),
    "gbfft_set_precision": (_int, [_vp, _int]),
    "gbfft_set_window": (_int, [_vp, _int]),
    "gbfft_set_noise": (_int, [_vp, ctypes.c_uint32, ctypes.c_float]),
    "gbfft_autotune": (_int, [_vp, _u64, _u64, _int, ctypes.POINTER(ctypes.c_double)]),
    "gbfft_launch_count": (_u64, [_vp]),
    "gbfft_version": (ctypes.c_char_p, []),
}

_lib = None
_lock = threading.Lock()


class GbfftError(RuntimeError):
    """A non-zero gbfft status; str() is the library's message."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status


def lib_path() -> str:
    return os.environ.get("GBFFT_LIB", LIB_PATH)


def load():
    """Load libgbfft.so (raises if it is absent -- there is no CPU path)."""
    global _lib
    with _lock:
        if _lib is None:
            path = lib_path()
            if not os.path.exists(path):
                raise RuntimeError(f"libgbfft.so not built ({path}); run gbfft.build.build()")
            L = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
        return _lib


def status_string(status: int) -> str:
    return load().gbfft_status_string(status).decode()


def is_available() -> bool:
    return bool(load().gbfft_is_available())


def _ptr(a) -> int:
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return int(a)


class Context:
    """Owns one gbfft_ctx (one device, one stream, a plan cache)."""

    def __init__(self, device: int = 0):
        self._L = load()
        h = _vp()
        st = self._L.gbfft_create(device, ctypes.byref(h))
        if st != OK:
            raise GbfftError(st, status_string(st))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._L.gbfft_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def last_error(self) -> str:
        return self._L.gbfft_last_error(self._h).decode()

    def _check(self, st: int):
        if st != OK:
            msg = self.last_error() or status_string(st)
            raise GbfftError(st, msg)

    def launch_count(self) -> int:
        return int(self._L.gbfft_launch_count(self._h))

    def set_precision(self, precision: int):
        self._check(self._L.gbfft_set_precision(self._h, precision))

    def set_window(self, window: int):
        """WINDOW_HANN: multiply every loaded input sample by the Hann window."""
        self._check(self._L.gbfft_set_window(self._h, window))

    def set_noise(self, seed: int, sigma: float):
        """Add the reference pipeline's PCG/Box-Muller noise on load (sigma 0: off)."""
        self._check(self._L.gbfft_set_noise(self._h, seed, sigma))

    def c2c_host(self, x: np.ndarray, direction: int = FORWARD, out: np.ndarray | None = None) -> np.ndarray:
        """Transform a [batch, n] complex64 host array (contiguous); returns out."""
        x = np.ascontiguousarray(x, dtype=np.complex64)
        if x.ndim == 1:
            x = x[None, :]
        if out is None:
            out = np.empty_like(x)
        b, n = x.shape
        self._check(self._L.gbfft_c2c_host(self._h, _ptr(x), _ptr(out), n, b, direction))
        return out

    def c2c_host_ptr(self, in_ptr: int, out_ptr: int, n: int, batch: int, direction: int):
        self._check(self._L.gbfft_c2c_host(self._h, in_ptr, out_ptr, n, batch, direction))

    def c2c_host_rows(self, rows, direction: int = FORWARD):
        """The reference's argument shape: a list of 1-D complex64 rows."""
        rows = [np.ascontiguousarray(r, dtype=np.complex64) for r in rows]
        outs = [np.empty_like(r) for r in rows]
        b = len(rows)
        in_p = (_vp * max(b, 1))(*[r.ctypes.data for r in rows])
        out_p = (_vp * max(b, 1))(*[o.ctypes.data for o in outs])
        lens = (_u64 * max(b, 1))(*[r.size for r in rows])
        self._check(self._L.gbfft_c2c_host_rows(self._h, in_p, lens, out_p, b, direction))
        return outs

    def c2c_device(self, d_in, d_out, n: int, batch: int, direction: int = FORWARD, stream=None):
        """Enqueue on device pointers (ints or tensors).  `stream` is a
        cudaStream_t as an int; None or 0 is the CUDA default stream."""
        s = 0 if stream is None else int(stream)
        self._check(self._L.gbfft_c2c_device(self._h, _ptr(d_in), _ptr(d_out), n, batch, direction, s or None))

    def bench_device(self, n: int, batch: int, direction: int = FORWARD, warmup: int = 3, iters: int = 20) -> float:
        sec = ctypes.c_double()
        self._check(self._L.gbfft_bench_device(self._h, n, batch, direction, warmup, iters, ctypes.byref(sec)))
        return sec.value

    def autotune(self, n: int, batch: int, direction: int = FORWARD) -> float:
        """Time every plan variant for (n, batch, direction, precision); the
        fastest serves later calls.  Returns its seconds per transform."""
        sec = ctypes.c_double()
        self._check(self._L.gbfft_autotune(self._h, n, batch, direction, ctypes.byref(sec)))
        return sec.value

    def ragged_plan(self, descs) -> "RaggedPlan":
        return RaggedPlan(self, descs)

    def ragged_device(self, d_in, d_out, capacity: int, descs, stream=None):
        d = ragged_descs(descs)
        s = 0 if stream is None else int(stream)
        self._check(self._L.gbfft_ragged_device(self._h, _ptr(d_in), _ptr(d_out), capacity, d.ctypes.data,
                                                len(d), s or None))


# struct gbfft_ragged_desc { uint64_t offset; uint32_t log2n; int32_t direction; }
RAGGED_DESC_DTYPE = np.dtype([("offset", "<u8"), ("log2n", "<u4"), ("direction", "<i4")])


def ragged_descs(descs) -> np.ndarray:
    """Descriptors as a contiguous gbfft_ragged_desc array.  Accepts such an
    array or an iterable of (offset, log2n, direction) tuples."""
    if isinstance(descs, np.ndarray) and descs.dtype == RAGGED_DESC_DTYPE:
        return np.ascontiguousarray(descs)
    return np.array([tuple(d) for d in descs], dtype=RAGGED_DESC_DTYPE)


class RaggedPlan:
    """A gbfft_ragged_plan: one persistent launch over mixed sizes/directions."""

    def __init__(self, ctx: Context, descs):
        self._ctx = ctx
        self._L = ctx._L
        self.descs = ragged_descs(descs)
        h = _vp()
        ctx._check(self._L.gbfft_ragged_plan_create(ctx.handle, self.descs.ctypes.data, len(self.descs),
                                                    ctypes.byref(h)))
        self._h = h

    def set(self, option: int, value: int):
        self._ctx._check(self._L.gbfft_ragged_plan_set(self._h, option, value))

    def execute(self, d_in, d_out, capacity: int, use_graph: bool = True, stream=None):
        s = 0 if stream is None else int(stream)
        self._ctx._check(self._L.gbfft_ragged_execute(self._h, _ptr(d_in), _ptr(d_out), capacity,
                                                      int(use_graph), s or None))

    def wait(self, stream=None):
        s = 0 if stream is None else int(stream)
        self._ctx._check(self._L.gbfft_ragged_wait(self._h, s or None))

    def launch_count(self) -> int:
        return int(self._L.gbfft_ragged_launch_count(self._h))

    def close(self):
        if getattr(self, "_h", None):
            self._L.gbfft_ragged_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


RAGGED_OPT_SPIN_LIMIT = 1
RAGGED_OPT_TEST_DROP_PRODUCERS = 2
RAGGED_OPT_LAG = 3
