"""gbfft: GB300-native batched power-of-two C2C FFT (Python side of the C ABI).

The transform itself lives in libgbfft.so (CUDA, sm_103a); this package only
builds and binds it.  Import it with ``wgls-rs-fft_gb300`` on sys.path.
"""
from ._lib import (ERR_CUDA, ERR_INVALID_ARGUMENT, ERR_INVALID_SIZE, ERR_LENGTH_MISMATCH, ERR_NO_DEVICE,
                   ERR_OUT_OF_MEMORY, ERR_TIMEOUT, ERR_UNSUPPORTED, FORWARD, INVERSE, OK, PREC_FP32,
                   PREC_TC_BF16X3, PREC_TC_BF16X6, PREC_TC_FP16, PREC_TC_TF32, WINDOW_HANN, WINDOW_NONE,
                   RAGGED_DESC_DTYPE, RAGGED_OPT_LAG, RAGGED_OPT_SPIN_LIMIT, RAGGED_OPT_TEST_DROP_PRODUCERS,
                   SIGNATURES, Context, GbfftError, RaggedPlan, is_available, lib_path, load, ragged_descs,
                   status_string)
from .build import LIB_PATH, build
from .gpu_fft import FftExecutor, GpuFft

__all__ = [
    "Context", "GbfftError", "GpuFft", "FftExecutor", "FORWARD", "INVERSE", "PREC_FP32", "OK",
    "ERR_INVALID_SIZE", "ERR_LENGTH_MISMATCH", "ERR_INVALID_ARGUMENT", "ERR_NO_DEVICE", "ERR_OUT_OF_MEMORY",
    "ERR_CUDA", "ERR_TIMEOUT", "ERR_UNSUPPORTED", "SIGNATURES", "build", "load", "lib_path", "LIB_PATH",
    "is_available", "status_string",
]
