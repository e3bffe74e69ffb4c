"""GPU: fused noise on load and the reference's noise -> FFT -> window -> IFFT
pipeline (examples/parallel_pipeline.rs) in two launches, eager and replayed
from a CUDA graph; checked against the oracle's restatement of the pipeline.

Gates: fused noise vs the oracle's float32 restatement, max |a - b| <= 1e-5
(the hash is exact; log/sqrt/sin/cos are different float32 libraries);
pipeline rel-L2 <= 2e-6 against FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    assert t.cuda.is_available()
    return t


@pytest.mark.parametrize("logn,batch", [(0, 4), (8, 5), (12, 3), (16, 2)])
def test_fused_noise_matches_reference_noise(lib_built, oracle, logn, batch):
    import gbfft
    n = 1 << logn
    with gbfft.Context(0) as ctx:
        ctx.set_noise(42, 0.1)
        zeros = np.zeros((batch, n), np.complex64)
        spec = ctx.c2c_host(zeros, gbfft.FORWARD)  # FFT of the noise alone
    want = oracle.fft64(oracle.ref_noise(batch, n, 42, 0.1))
    assert oracle.rel_l2(spec, want) <= 2e-6
    with gbfft.Context(0) as ctx:  # the noise itself, through an N=1 identity transform
        ctx.set_noise(7, 0.25)
        got = ctx.c2c_host(np.zeros((n * batch, 1), np.complex64), gbfft.FORWARD).reshape(-1)
    # N = 1 transforms: row index = sample index, element index 0
    want1 = oracle.ref_noise(n * batch, 1, 7, 0.25).reshape(-1)
    assert oracle.max_abs_err(got, want1) <= 1e-5


@pytest.mark.parametrize("logn,batch", [(10, 8), (12, 16), (15, 4)])
def test_pipeline_eager_and_graph(lib_built, oracle, torch, logn, batch):
    from gbfft import signals
    from gbfft.pipeline import SpectralPipeline
    n = 1 << logn
    p = SpectralPipeline(n, batch, slots=2, seed=42, sigma=0.1)
    xs = [signals.uniform_c64(batch, n, seed=s) for s in (1, 2)]
    for i, x in enumerate(xs):
        p.inputs[i].copy_(torch.from_numpy(x))
    p.run_eager()
    torch.cuda.synchronize()
    eager = [o.cpu().numpy() for o in p.outputs]
    for i, x in enumerate(xs):
        assert oracle.rel_l2(eager[i], oracle.ref_pipeline(x, 42, 0.1)) <= 2e-6
    for o in p.outputs:
        o.zero_()
    p.capture()
    p.replay()
    torch.cuda.synchronize()
    for i in range(2):
        assert np.array_equal(p.outputs[i].cpu().numpy(), eager[i])
    p.close()


def test_pipeline_host_frames_six_slots(lib_built, oracle, torch):
    """The reference's loop (examples/parallel_pipeline.rs:696-735): 14 host
    frames of N = 1024 x 8 through six slots in flight, frame f with noise
    seed f; every output against the FP64 pipeline, in frame order, and the
    same bits as one frame through the pipeline on its own."""
    from gbfft import signals
    from gbfft.pipeline import SpectralPipeline
    n, batch, nframes = 1024, 8, 14
    frames = [signals.uniform_c64(batch, n, seed=100 + f) for f in range(nframes)]
    p = SpectralPipeline(n, batch, slots=6, sigma=0.1)
    outs = p.run_frames(frames)
    assert len(outs) == nframes
    for f, (x, y) in enumerate(zip(frames, outs)):
        assert oracle.rel_l2(y, oracle.ref_pipeline(x, f, 0.1)) <= 2e-6, f
    again = p.run_frames(frames[5:6], seed_base=5)
    assert np.array_equal(again[0], outs[5])
    p.close()


def test_noise_argument_checks(lib_built):
    import gbfft
    with gbfft.Context(0) as ctx:
        with pytest.raises(gbfft.GbfftError) as e:
            ctx.set_noise(1, -1.0)
        assert e.value.status == gbfft.ERR_INVALID_ARGUMENT
        ctx.set_noise(1, 0.0)
        x = np.ones((1, 4), np.complex64)
        assert np.allclose(ctx.c2c_host(x, gbfft.FORWARD)[0], [4, 0, 0, 0])
