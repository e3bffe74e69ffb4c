"""GPU: the allocation-free entry point gbfft_c2c_device_noalloc.

It serves callers that may not allocate GPU memory (code inside another
library's allocator hook, a pool that owns all device memory, latency-critical
paths): it runs the two-pass transform with the library's built-in scratch
array instead of a workspace from cudaMalloc.  Checked here through the C ABI
against the regular device entry point, on two calls in a row, with the
suite's tolerances, and against the FP64 oracle; and that, once each size has
run once (its kernels loaded), further calls leave the device's free memory
unchanged.  This file is collected last so that a stop-at-first-failure run
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_REL_L2 = 2e-6  # the FP32 form's tolerance in every GPU test


def _noalloc(L, x, y, n, batch, direction, stream):
    return L.gbfft_c2c_device_noalloc(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), n, batch,
                                      direction, ctypes.c_void_p(stream) if stream else None)


def _rel(a, b):
    import torch
    return (torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b)).item()


@pytest.mark.parametrize("logn,batch", [(15, 128), (16, 64), (18, 16), (20, 4)])
def test_noalloc_matches_device_entry_two_calls(gpu_ctx, oracle, logn, batch):
    torch = pytest.importorskip("torch")
    import gbfft
    from gbfft import signals
    L = gbfft.load()
    n = 1 << logn
    s = torch.cuda.current_stream().cuda_stream
    x1 = signals.normal_c64_torch(batch, n, seed=31)
    x2 = signals.uniform_c64_torch(batch, n, seed=32)
    for x, direction in ((x1, gbfft.FORWARD), (x2, gbfft.INVERSE)):  # two calls in a row
        want = torch.empty_like(x)
        gpu_ctx.c2c_device(x, want, n, batch, direction, stream=s)
        got = torch.empty_like(x)
        assert _noalloc(L, x, got, n, batch, direction, s) == gbfft.OK
        torch.cuda.synchronize()
        assert _rel(got, want) <= TOL_REL_L2
        # and against the FP64 oracle on three rows (first, middle, last)
        rows = [0, batch // 2, batch - 1]
        ref = oracle.fft64(x[rows].cpu().numpy(), inverse=(direction == gbfft.INVERSE))
        assert oracle.rel_l2(got[rows].cpu().numpy(), ref) <= TOL_REL_L2


def test_noalloc_leaves_free_memory_unchanged(gpu_ctx):
    """After one call of each size (the first call sets up, and the first
    launch of each kernel may load its code), further calls of every size and
    both directions do not change the device's free memory."""
    torch = pytest.importorskip("torch")
    import gbfft
    from gbfft import signals
    L = gbfft.load()
    s = torch.cuda.current_stream().cuda_stream
    shapes = [(15, 64), (16, 32), (17, 16), (18, 8), (19, 4), (20, 2)]
    bufs = [(signals.uniform_c64_torch(b, 1 << lg, seed=34 + lg), torch.empty(b, 1 << lg, dtype=torch.complex64,
                                                                           device="cuda")) for lg, b in shapes]
    for (lg, b), (x, y) in zip(shapes, bufs):
        for direction in (gbfft.FORWARD, gbfft.INVERSE):
            assert _noalloc(L, x, y, 1 << lg, b, direction, s) == gbfft.OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        for (lg, b), (x, y) in zip(shapes, bufs):
            for direction in (gbfft.FORWARD, gbfft.INVERSE):
                assert _noalloc(L, x, y, 1 << lg, b, direction, s) == gbfft.OK
                assert _noalloc(L, y, y, 1 << lg, b, direction, s) == gbfft.OK  # in place
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def test_noalloc_in_place_and_limits(gpu_ctx):
    torch = pytest.importorskip("torch")
    import gbfft
    from gbfft import signals
    L = gbfft.load()
    n, batch = 1 << 16, 8
    s = torch.cuda.current_stream().cuda_stream
    x = signals.uniform_c64_torch(batch, n, seed=33)
    want = torch.empty_like(x)
    gpu_ctx.c2c_device(x, want, n, batch, gbfft.FORWARD, stream=s)
    y = x.clone()
    assert _noalloc(L, y, y, n, batch, gbfft.FORWARD, s) == gbfft.OK  # in place
    torch.cuda.synchronize()
    assert _rel(y, want) <= TOL_REL_L2
    # limits: n * batch above the 2^22-sample scratch, n outside 2^15..2^20
    assert _noalloc(L, x, y, n, (1 << 22) // n + 1, gbfft.FORWARD, s) == gbfft.ERR_UNSUPPORTED
    assert _noalloc(L, x, y, 1 << 14, 4, gbfft.FORWARD, s) == gbfft.ERR_UNSUPPORTED
    assert _noalloc(L, x, y, 1 << 21, 1, gbfft.FORWARD, s) == gbfft.ERR_UNSUPPORTED
    assert _noalloc(L, x, y, 3 << 15, 1, gbfft.FORWARD, s) == gbfft.ERR_INVALID_SIZE
    assert _noalloc(L, x, y, n, batch, 0, s) == gbfft.ERR_INVALID_ARGUMENT
