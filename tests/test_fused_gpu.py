"""GPU: the fused pass pairs (two global passes in one persistent launch,
intermediate read back from L2): both passes of N = 2^15 .. 2^20, and the last
two passes of N = 2^21 .. 2^26.

The form runs the same tile arithmetic as the two-launch form, so its output
must be bit-identical to it; both are also checked against FP64 at
rel-L2 <= 2e-6.  Variants are forced through the on-disk tuning cache
(GBFFT_AUTOTUNE_CACHE).  Covered: batches smaller than, equal to and far
larger than the producer/consumer lag, both directions, repeated launches
(the kernel clears its own counters), two streams, noise on load, and the
in-place fallback."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_REL_L2 = 2e-6


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    assert t.cuda.is_available()
    return t


def _force(tmp_path, monkeypatch, logn, batch, fused, max_logr=10, loge=4):
    import gbfft
    lines = []
    for d in (gbfft.FORWARD, gbfft.INVERSE):
        lines.append(json.dumps({"arch": "sm_103", "logn": logn, "precision": 0, "direction": d,
                                 "batch_log2": batch.bit_length() - 1, "max_logr": max_logr, "persistent": 0,
                                 "fused": int(fused), "tile": 0, "loge": loge, "seconds": 1.0}))
    cache = tmp_path / f"tune_{int(fused)}_{loge}.jsonl"
    cache.write_text("\n".join(lines) + "\n")
    monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))


def _run(torch, x, direction, fused, tmp_path, monkeypatch, repeats=1, noise=None, loge=4):
    import gbfft
    batch, n = x.shape
    _force(tmp_path, monkeypatch, n.bit_length() - 1, batch, fused, loge=loge)
    dx = torch.from_numpy(x).cuda()
    outs = []
    with gbfft.Context(0) as ctx:
        if noise:
            ctx.set_noise(*noise)
        for _ in range(repeats):
            dy = torch.full_like(dx, float("nan"))
            ctx.c2c_device(dx, dy, n, batch, direction)
            torch.cuda.synchronize()
            outs.append(dy.cpu().numpy())
        launches = ctx.launch_count()
    return outs, launches


@pytest.mark.parametrize("logn,batch", [(15, 1), (15, 37), (16, 3), (16, 200), (17, 5), (18, 9), (19, 2), (20, 3)])
def test_fused_matches_two_launches_and_fp64(torch, oracle, lib_built, tmp_path, monkeypatch, logn, batch):
    import gbfft
    from gbfft import signals
    x = signals.normal_c64(batch, 1 << logn, seed=300 + logn)
    for d, inv in ((gbfft.FORWARD, False), (gbfft.INVERSE, True)):
        (yf,), lf = _run(torch, x, d, True, tmp_path, monkeypatch)
        (yp,), lp = _run(torch, x, d, False, tmp_path, monkeypatch)
        assert lf == 1 and lp == 2  # one launch against two
        assert np.array_equal(yf, yp)
        assert oracle.rel_l2(yf, oracle.fft64(x, inverse=inv)) <= TOL_REL_L2


def test_fused_repeated_launches_reset_counters(torch, lib_built, tmp_path, monkeypatch):
    import gbfft
    from gbfft import signals
    x = signals.uniform_c64(96, 1 << 16, seed=310)
    outs, launches = _run(torch, x, gbfft.FORWARD, True, tmp_path, monkeypatch, repeats=5)
    assert launches == 5
    for y in outs[1:]:
        assert np.array_equal(y, outs[0])


def test_fused_two_streams(torch, oracle, lib_built, tmp_path, monkeypatch):
    import gbfft
    from gbfft import signals
    n, batch = 1 << 17, 24
    _force(tmp_path, monkeypatch, 17, batch, True)
    xs = [signals.normal_c64(batch, n, seed=320 + i) for i in range(2)]
    dxs = [torch.from_numpy(x).cuda() for x in xs]
    dys = [torch.empty_like(d) for d in dxs]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    torch.cuda.synchronize()
    with gbfft.Context(0) as ctx:
        for rep in range(3):
            for i in range(2):
                ctx.c2c_device(dxs[i], dys[i], n, batch, gbfft.FORWARD, stream=streams[i].cuda_stream)
        torch.cuda.synchronize()
    for i in range(2):
        assert oracle.rel_l2(dys[i].cpu().numpy(), oracle.fft64(xs[i])) <= TOL_REL_L2


def test_fused_noise_on_load(torch, lib_built, tmp_path, monkeypatch):
    import gbfft
    x = np.zeros((12, 1 << 15), np.complex64)
    (yf,), _ = _run(torch, x, gbfft.FORWARD, True, tmp_path, monkeypatch, noise=(9, 0.5))
    (yp,), _ = _run(torch, x, gbfft.FORWARD, False, tmp_path, monkeypatch, noise=(9, 0.5))
    assert np.array_equal(yf, yp) and np.abs(yf).max() > 0


def test_fused_in_place_falls_back(torch, oracle, lib_built, tmp_path, monkeypatch):
    import gbfft
    from gbfft import signals
    n, batch = 1 << 16, 7
    _force(tmp_path, monkeypatch, 16, batch, True)
    x = signals.normal_c64(batch, n, seed=330)
    d = torch.from_numpy(x).cuda()
    with gbfft.Context(0) as ctx:
        ctx.c2c_device(d, d, n, batch, gbfft.INVERSE)
        torch.cuda.synchronize()
        assert ctx.launch_count() == 2
    assert oracle.rel_l2(d.cpu().numpy(), oracle.fft64(x, inverse=True)) <= TOL_REL_L2


# ---- last two passes of a three-pass transform (radices 2^(L-16), 256, 256) ----

@pytest.mark.parametrize("logn,batch", [(21, 3), (22, 2), (23, 1), (24, 1)])
def test_fused_last_two_of_three_vs_fp64(torch, oracle, lib_built, tmp_path, monkeypatch, logn, batch):
    import gbfft
    from gbfft import signals
    x = signals.normal_c64(batch, 1 << logn, seed=340 + logn)
    for d, inv in ((gbfft.FORWARD, False), (gbfft.INVERSE, True)):
        (yf,), lf = _run(torch, x, d, True, tmp_path, monkeypatch)
        (yp,), lp = _run(torch, x, d, False, tmp_path, monkeypatch)
        assert lf == 2 and lp == 3  # first pass + the fused pair, against three launches
        want = oracle.fft64(x, inverse=inv)
        assert oracle.rel_l2(yf, want) <= TOL_REL_L2
        assert oracle.rel_l2(yp, want) <= TOL_REL_L2


def test_fused_last_two_of_three_in_place_and_repeated(torch, oracle, lib_built, tmp_path, monkeypatch):
    import gbfft
    from gbfft import signals
    n, batch = 1 << 22, 3
    _force(tmp_path, monkeypatch, 22, batch, True)
    x = signals.uniform_c64(batch, n, seed=350)
    want = oracle.fft64(x)
    with gbfft.Context(0) as ctx:
        d = torch.from_numpy(x).cuda()
        ctx.c2c_device(d, d, n, batch, gbfft.FORWARD)  # in place: the first pass writes the workspace
        torch.cuda.synchronize()
        assert oracle.rel_l2(d.cpu().numpy(), want) <= TOL_REL_L2
        dx = torch.from_numpy(x).cuda()
        outs = []
        for _ in range(3):  # the pair kernel clears its own counters
            dy = torch.full_like(dx, float("nan"))
            ctx.c2c_device(dx, dy, n, batch, gbfft.FORWARD)
            torch.cuda.synchronize()
            outs.append(dy.cpu().numpy())
        assert ctx.launch_count() == 8
    for y in outs:
        assert np.array_equal(y, outs[0])
    assert oracle.rel_l2(outs[0], want) <= TOL_REL_L2


def test_fused_last_two_of_three_full_size_roundtrip(torch, lib_built):
    """N = 2^26 (one transform, 512 MB) through the default plan: roundtrip and
    Parseval (the FP64 oracle of a 2^26-point transform is too slow here)."""
    import gbfft
    from gbfft import signals
    n = 1 << 26
    x = signals.normal_c64_torch(1, n, seed=360)
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    with gbfft.Context(0) as ctx:
        ctx.c2c_device(x, y, n, 1, gbfft.FORWARD)
        ctx.c2c_device(y, z, n, 1, gbfft.INVERSE)
        torch.cuda.synchronize()
        assert ctx.launch_count() == 4
    rt = (torch.linalg.vector_norm(z - x) / torch.linalg.vector_norm(x)).item()
    assert rt < 1e-6
    ex = torch.linalg.vector_norm(x.to(torch.complex128)).item() ** 2
    ey = torch.linalg.vector_norm(y.to(torch.complex128)).item() ** 2 / n
    assert abs(ey / ex - 1) < 1e-5


@pytest.mark.parametrize("logn,batch", [(13, 5), (13, 64), (14, 3), (14, 33)])
def test_fused_radix128_pair_for_single_pass_sizes(torch, oracle, lib_built, tmp_path, monkeypatch, logn, batch):
    """N = 2^13, 2^14 as a fused two-pass transform of radix-128 tiles (an
    autotuner candidate beside the single-pass kernels)."""
    import gbfft
    from gbfft import signals
    x = signals.normal_c64(batch, 1 << logn, seed=370 + logn)
    for d, inv in ((gbfft.FORWARD, False), (gbfft.INVERSE, True)):
        (yf,), lf = _run(torch, x, d, True, tmp_path, monkeypatch)
        assert lf == 1
        assert oracle.rel_l2(yf, oracle.fft64(x, inverse=inv)) <= TOL_REL_L2


@pytest.mark.parametrize("logn,batch", [(15, 3), (16, 7), (17, 1), (17, 33), (18, 5), (18, 40), (19, 3), (20, 2),
                                        (20, 9)])
def test_fused_32_samples_per_thread(torch, oracle, lib_built, tmp_path, monkeypatch, logn, batch):
    """The pass pair with 32 samples a thread (radix-32 sub-passes: a
    radix-2^9 pass as 32 x 16 instead of 16 x 16 x 2, 2^10 as 32 x 32 instead
    of 16 x 16 x 4, 2^8 as 32 x 8, 2^7 as 32 x 4), with its own sub-pass tables: FP64 gate, agreement with
    the 16-sample pair to FP32 rounding, repeated launches, noise on load."""
    import gbfft
    from gbfft import signals
    x = signals.normal_c64(batch, 1 << logn, seed=340 + logn + batch)
    for d, inv in ((gbfft.FORWARD, False), (gbfft.INVERSE, True)):
        (y5, y5b), l5 = _run(torch, x, d, True, tmp_path, monkeypatch, repeats=2, loge=5)
        (y4,), _ = _run(torch, x, d, True, tmp_path, monkeypatch, loge=4)
        assert l5 == 2  # one launch a transform
        assert np.array_equal(y5, y5b)
        assert oracle.rel_l2(y5, oracle.fft64(x, inverse=inv)) <= TOL_REL_L2
        assert oracle.rel_l2(y5, y4) <= 1e-6
    z = np.zeros((3, 1 << logn), np.complex64)
    (n5,), _ = _run(torch, z, gbfft.FORWARD, True, tmp_path, monkeypatch, noise=(11, 0.5), loge=5)
    (n4,), _ = _run(torch, z, gbfft.FORWARD, True, tmp_path, monkeypatch, noise=(11, 0.5), loge=4)
    assert np.abs(n4).max() > 0 and oracle.rel_l2(n5, n4) <= 1e-6
