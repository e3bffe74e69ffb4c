"""GPU: the Hann window fused into the transform's load (gbfft_set_window),
against the FP64 oracle applied to the explicitly windowed signal, and the
reference's windowed-FFT tests (tests/windowed_fft_test.rs) on the fused path.
Gate: relative L2 <= 2e-6 (FP32 and FP16-split forms)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 2e-6


@pytest.fixture()
def wctx(lib_built):
    import gbfft
    ctx = gbfft.Context(0)
    ctx.set_window(gbfft.WINDOW_HANN)
    yield ctx
    ctx.close()


@pytest.mark.parametrize("logn,batch", [(0, 3), (4, 5), (10, 8), (12, 33), (13, 4), (14, 2), (16, 4), (20, 1),
                                        (22, 1)])
def test_hann_fused_matches_explicit(wctx, oracle, logn, batch):
    import gbfft
    from gbfft import signals
    n = 1 << logn
    x = signals.normal_c64(batch, n, seed=90 + logn)
    w = signals.hann_window(n).astype(np.float64)
    xw = x.astype(np.complex128) * w[None, :]
    for d, inv in ((gbfft.FORWARD, False), (gbfft.INVERSE, True)):
        y = wctx.c2c_host(x, d)
        assert oracle.rel_l2(y, oracle.fft64(xw, inverse=inv)) <= TOL, (logn, inv)


def test_hann_fused_split_form(wctx, oracle):
    import gbfft
    from gbfft import signals
    wctx.set_precision(gbfft.PREC_TC_FP16)
    n = 1 << 16
    x = signals.normal_c64(4, n, seed=99)
    xw = x.astype(np.complex128) * signals.hann_window(n).astype(np.float64)[None, :]
    assert oracle.rel_l2(wctx.c2c_host(x, gbfft.FORWARD), oracle.fft64(xw)) <= TOL


def test_reference_windowed_tests_fused(wctx, lib_built):
    """tests/windowed_fft_test.rs with the window applied by the kernel:
    roundtrip through an unwindowed inverse < 1e-3, power ratio in (0.1, 10),
    peaks at bins 10 and 50 (N = 2048)."""
    import gbfft
    from conftest import golden
    g = golden("ref_signals.npz")
    tone, hann = g["tone2048"][None, :], g["hann2048"][None, :]
    spec = wctx.c2c_host(tone, gbfft.FORWARD)
    with gbfft.Context(0) as plain:
        rec = plain.c2c_host(spec, gbfft.INVERSE)
        orig = plain.c2c_host(tone, gbfft.FORWARD)
    assert np.max(np.abs(rec - hann)) < 1e-3
    ratio = np.sum(np.abs(spec) ** 2) / np.sum(np.abs(orig) ** 2)
    assert 0.1 < ratio < 10.0
    p = np.abs(spec[0]) ** 2
    peaks = [i for i in range(1, 1024) if p[i] > p[i - 1] and p[i] > p[i + 1] and p[i] > 10.0]
    assert 10 in peaks and 50 in peaks


def test_window_limits(wctx):
    import gbfft
    with pytest.raises(gbfft.GbfftError) as e:
        wctx.set_window(5)
    assert e.value.status == gbfft.ERR_INVALID_ARGUMENT
    with pytest.raises(gbfft.GbfftError) as e:  # window tables stop at 2^24
        wctx.c2c_host(np.zeros((1, 1 << 25), np.complex64), gbfft.FORWARD)
    assert e.value.status == gbfft.ERR_UNSUPPORTED
    wctx.set_window(gbfft.WINDOW_NONE)
    x = np.ones((1, 8), np.complex64)
    assert np.allclose(wctx.c2c_host(x, gbfft.FORWARD)[0], [8, 0, 0, 0, 0, 0, 0, 0], atol=1e-6)


@pytest.mark.parametrize("logn,batch", [(15, 6), (16, 40), (18, 3), (20, 2)])
def test_hann_fused_two_pass_device_entry(lib_built, oracle, logn, batch):
    """Out of place on the device, N = 2^15..2^20 runs the fused two-pass
    launch; the window is applied by its first-pass tiles."""
    torch = pytest.importorskip("torch")
    import gbfft
    from gbfft import signals
    n = 1 << logn
    x = signals.normal_c64(batch, n, seed=95 + logn)
    xw = x.astype(np.complex128) * signals.hann_window(n).astype(np.float64)[None, :]
    dx = torch.from_numpy(x).cuda()
    dy = torch.empty_like(dx)
    with gbfft.Context(0) as ctx:
        ctx.set_window(gbfft.WINDOW_HANN)
        for d, inv in ((gbfft.FORWARD, False), (gbfft.INVERSE, True)):
            l0 = ctx.launch_count()
            ctx.c2c_device(dx, dy, n, batch, d)
            torch.cuda.synchronize()
            assert ctx.launch_count() - l0 == 1  # the fused form ran
            assert oracle.rel_l2(dy.cpu().numpy(), oracle.fft64(xw, inverse=inv)) <= TOL, (logn, inv)
