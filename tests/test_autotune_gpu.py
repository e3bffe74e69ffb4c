"""GPU: the autotuner and every plan variant it chooses between.

Each variant (global-pass split cap, plain or persistent tile-loop kernels,
samples -- hence transforms -- per CTA of the single-pass kernel) is
forced through the documented on-disk cache (GBFFT_AUTOTUNE_CACHE) and checked
against FP64 at rel-L2 <= 2e-6; the tuner itself must return a positive time,
keep results correct and append its choice to the cache file."""
import json
import os

import pytest

pytestmark = pytest.mark.gpu

TOL_REL_L2 = 2e-6


def _cache_line(logn, batch, direction, max_logr, persistent, precision=0, tile=0, loge=None):
    d = {"arch": "sm_103", "logn": logn, "precision": precision, "direction": direction,
         "batch_log2": batch.bit_length() - 1, "max_logr": max_logr, "persistent": persistent,
         "fused": 0, "tile": tile}
    if loge is not None:  # lines without the key (older caches) mean 16 samples a thread
        d["loge"] = loge
    d["seconds"] = 1.0
    return json.dumps(d)


@pytest.mark.parametrize("logn,batch,max_logr,persistent", [
    (12, 64, 10, 1), (13, 64, 10, 0), (13, 64, 10, 1), (14, 32, 10, 0), (14, 32, 10, 1),
    (15, 16, 10, 1), (16, 16, 8, 0), (16, 16, 8, 1), (18, 4, 9, 1), (18, 4, 7, 0),
    (20, 2, 10, 1), (20, 2, 9, 0), (20, 2, 7, 1), (22, 1, 8, 1), (22, 1, 10, 0),
])
def test_forced_variant_correct(tmp_path, monkeypatch, oracle, lib_built, logn, batch, max_logr, persistent):
    import gbfft
    from gbfft import signals
    cache = tmp_path / "tune.jsonl"
    cache.write_text(_cache_line(logn, batch, gbfft.FORWARD, max_logr, persistent) + "\n" +
                     _cache_line(logn, batch, gbfft.INVERSE, max_logr, persistent) + "\n")
    monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
    x = signals.normal_c64(batch, 1 << logn, seed=70 + logn)
    with gbfft.Context(0) as ctx:
        for d, inv in ((gbfft.FORWARD, False), (gbfft.INVERSE, True)):
            y = ctx.c2c_host(x, d)
            assert oracle.rel_l2(y, oracle.fft64(x, inverse=inv)) <= TOL_REL_L2


@pytest.mark.parametrize("logn,batch", [(13, 512), (16, 64), (20, 4)])
def test_autotune_choice_is_used_and_cached(tmp_path, monkeypatch, oracle, lib_built, logn, batch):
    import gbfft
    from gbfft import signals
    cache = tmp_path / "tune.jsonl"
    monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
    with gbfft.Context(0) as ctx:
        sec = ctx.autotune(1 << logn, batch, gbfft.FORWARD)
        assert sec > 0
        x = signals.uniform_c64(batch, 1 << logn, seed=80)
        y = ctx.c2c_host(x, gbfft.FORWARD)
        assert oracle.rel_l2(y, oracle.fft64(x)) <= TOL_REL_L2
    lines = [json.loads(l) for l in cache.read_text().splitlines()]
    assert len(lines) == 1 and lines[0]["logn"] == logn and lines[0]["seconds"] > 0
    with gbfft.Context(0) as ctx2:  # the cache is read back by a new context
        y2 = ctx2.c2c_host(x, gbfft.FORWARD)
        assert oracle.rel_l2(y2, y) <= TOL_REL_L2


def test_autotune_on_first_use(monkeypatch, oracle, lib_built):
    import gbfft
    from gbfft import signals
    monkeypatch.setenv("GBFFT_AUTOTUNE", "1")
    monkeypatch.delenv("GBFFT_AUTOTUNE_CACHE", raising=False)
    with gbfft.Context(0) as ctx:
        x = signals.uniform_c64(8, 1 << 17, seed=81)
        y = ctx.c2c_host(x, gbfft.INVERSE)
        assert oracle.rel_l2(y, oracle.fft64(x, inverse=True)) <= TOL_REL_L2


@pytest.mark.parametrize("logn", [6, 8, 10, 11])
@pytest.mark.parametrize("tile,persistent", [(11, 0), (13, 0), (13, 1)])
def test_forced_transforms_per_cta(tmp_path, monkeypatch, oracle, lib_built, logn, tile, persistent):
    """Single-pass kernels moving 2^11 or 2^13 samples per CTA (half or twice
    the default number of transforms per CTA), batch not a multiple of it."""
    import gbfft
    from gbfft import signals
    batch = (1 << (14 - logn)) + 3
    cache = tmp_path / "tune.jsonl"
    cache.write_text("\n".join(_cache_line(logn, batch, d, 10, persistent, tile=tile)
                               for d in (gbfft.FORWARD, gbfft.INVERSE)) + "\n")
    monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
    x = signals.normal_c64(batch, 1 << logn, seed=500 + logn + tile)
    with gbfft.Context(0) as ctx:
        for d, inv in ((gbfft.FORWARD, False), (gbfft.INVERSE, True)):
            y = ctx.c2c_host(x, d)
            assert oracle.rel_l2(y, oracle.fft64(x, inverse=inv)) <= TOL_REL_L2


@pytest.mark.parametrize("logn", [13, 14])
@pytest.mark.parametrize("persistent", [0, 1])
@pytest.mark.parametrize("batch", [1, 37, 333])
def test_forced_32_samples_per_thread(tmp_path, monkeypatch, oracle, lib_built, logn, persistent, batch):
    """Single-pass N = 2^13 / 2^14 with 32 samples a thread (radix-32
    sub-passes 32 x 32 x 8 and 32 x 32 x 16: two shared-memory exchanges
    instead of three): FP64 gate, the reference path's 1e-3 gate, roundtrip;
    batches below, near and above the persistent grid."""
    import gbfft
    from gbfft import signals
    cache = tmp_path / "tune.jsonl"
    cache.write_text("\n".join(_cache_line(logn, batch, d, 10, persistent, loge=5)
                               for d in (gbfft.FORWARD, gbfft.INVERSE)) + "\n")
    monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
    x = signals.normal_c64(batch, 1 << logn, seed=900 + logn + batch)
    with gbfft.Context(0) as ctx:
        y = ctx.c2c_host(x, gbfft.FORWARD)
        assert oracle.rel_l2(y, oracle.fft64(x)) <= TOL_REL_L2
        k = min(batch, 4)  # the reference path (a CPU restatement) on a few rows
        assert oracle.max_abs_err(y[:k], oracle.ref_fft(x[:k])) <= 1e-3
        z = ctx.c2c_host(y, gbfft.INVERSE)
        assert oracle.rel_l2(z, oracle.fft64(y, inverse=True)) <= TOL_REL_L2
        assert oracle.rel_l2(z, x) <= 1e-6


@pytest.mark.parametrize("logn", [13, 14])
def test_32_samples_per_thread_matches_16_with_load_ops(tmp_path, monkeypatch, oracle, lib_built, logn):
    """The window and the pipeline noise applied on load give the same
    transform in both thread layouts (to FP32 rounding)."""
    import gbfft
    from gbfft import signals
    batch = 6
    x = signals.uniform_c64(batch, 1 << logn, seed=950 + logn)
    outs = []
    for loge in (4, 5):
        cache = tmp_path / f"tune_{loge}.jsonl"
        cache.write_text("\n".join(_cache_line(logn, batch, d, 10, 0, loge=loge)
                                   for d in (gbfft.FORWARD, gbfft.INVERSE)) + "\n")
        monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
        with gbfft.Context(0) as ctx:
            ctx.set_window(gbfft.WINDOW_HANN)
            ctx.set_noise(7, 0.1)
            outs.append([ctx.c2c_host(x, d) for d in (gbfft.FORWARD, gbfft.INVERSE)])
    for a, b in zip(*outs):
        assert oracle.rel_l2(b, a) <= 1e-6
    # the window alone against FP64 of the windowed input
    with gbfft.Context(0) as ctx:
        ctx.set_window(gbfft.WINDOW_HANN)
        w = signals.hann_window(1 << logn)
        y = ctx.c2c_host(x, gbfft.FORWARD)
        assert oracle.rel_l2(y, oracle.fft64(x * w[None, :])) <= TOL_REL_L2


@pytest.mark.parametrize("logn", [25, 26])
def test_three_pass_first_pass_32_samples(tmp_path, monkeypatch, oracle, lib_built, logn):
    """N = 2^25 / 2^26 as (L-16, 8, 8) with the first pass (radix 2^9 / 2^10)
    run with 32 samples a thread: agrees with the 16-sample plan to FP32
    rounding in both directions; 2^25 also against numpy's FP64 FFT."""
    import numpy as np

    import gbfft
    from gbfft import signals
    x = signals.normal_c64(1, 1 << logn, seed=990 + logn)
    outs = {}
    for loge in (4, 5):
        cache = tmp_path / f"tune_{loge}.jsonl"
        lines = []
        for d in (gbfft.FORWARD, gbfft.INVERSE):
            line = json.loads(_cache_line(logn, 1, d, 10, 0, loge=loge))
            line["fused"] = 1
            lines.append(json.dumps(line))
        cache.write_text("\n".join(lines) + "\n")
        monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
        with gbfft.Context(0) as ctx:
            outs[loge] = [ctx.c2c_host(x, d) for d in (gbfft.FORWARD, gbfft.INVERSE)]
    for a, b in zip(outs[4], outs[5]):
        assert oracle.rel_l2(b, a) <= 1e-6
    if logn == 25:
        ref = np.fft.fft(x.astype(np.complex128), axis=1)
        assert oracle.rel_l2(outs[5][0], ref) <= TOL_REL_L2


@pytest.mark.parametrize("logn,batch,loge,persistent", [
    (25, 2, 5, 0), (25, 2, 4, 0), (26, 1, 5, 0), (26, 1, 4, 0), (25, 1, 5, 1)])
def test_three_pass_first_pass_8_columns(tmp_path, monkeypatch, oracle, lib_built, logn, batch, loge, persistent):
    """N = 2^25 / 2^26 as (L-16, 8, 8) with the radix-2^9 / 2^10 first pass on
    8 columns a CTA (plan tile 3; two CTAs per SM) instead of 16.  Each column's
    arithmetic is unchanged, so both directions give the same bits as the
    16-column first pass; 2^25 also meets the FP64 gate."""
    import numpy as np

    import gbfft
    from gbfft import signals
    x = signals.normal_c64(batch, 1 << logn, seed=1300 + logn + loge)
    outs = {}
    for tile in (0, 3):
        cache = tmp_path / f"tune_{tile}.jsonl"
        lines = []
        for d in (gbfft.FORWARD, gbfft.INVERSE):
            line = json.loads(_cache_line(logn, batch, d, 10, persistent, tile=tile, loge=loge))
            line["fused"] = 1
            lines.append(json.dumps(line))
        cache.write_text("\n".join(lines) + "\n")
        monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
        with gbfft.Context(0) as ctx:
            outs[tile] = [ctx.c2c_host(x, d) for d in (gbfft.FORWARD, gbfft.INVERSE)]
    for a, b in zip(outs[0], outs[3]):
        assert np.array_equal(a, b)
    if logn == 25 and persistent == 0:
        ref = np.fft.fft(x.astype(np.complex128), axis=1)
        assert oracle.rel_l2(outs[3][0], ref) <= TOL_REL_L2


@pytest.mark.parametrize("loge,persistent", [(5, 0), (4, 0), (5, 1)])
@pytest.mark.parametrize("logn,batch", [(25, 2), (26, 1)])
def test_three_pass_first_pass_tma(tmp_path, monkeypatch, oracle, lib_built, logn, batch, loge, persistent):
    """The 8-column first pass of N = 2^25 / 2^26 (32 or 16 samples a thread)
    with its input tile brought into shared memory by the tensor memory
    accelerator (tiled copies of a [256 rows][8 columns] box of a 3-D tensor
    map; plan key "tma": 1; persistent: a tile loop that prefetches the next
    tile's boxes into L2) against the same pass with 8-byte loads ("tma": 0):
    the same bits in both directions, and the FP64 gate."""
    import numpy as np

    import gbfft
    from gbfft import signals
    x = signals.normal_c64(batch, 1 << logn, seed=1350 + logn)
    outs = {}
    for tma in (0, 1):
        cache = tmp_path / f"tune_tma{tma}_{loge}_{persistent}.jsonl"
        lines = []
        for d in (gbfft.FORWARD, gbfft.INVERSE):
            line = json.loads(_cache_line(logn, batch, d, 10, persistent if tma else 0, tile=3, loge=loge))
            line["fused"] = 1
            line["tma"] = tma
            line["seconds"] = line.pop("seconds")  # key order as the library writes it
            lines.append(json.dumps(line))
        cache.write_text("\n".join(lines) + "\n")
        monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
        with gbfft.Context(0) as ctx:
            outs[tma] = [ctx.c2c_host(x, d) for d in (gbfft.FORWARD, gbfft.INVERSE)]
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    for y, inv in zip(outs[1], (False, True)):
        assert oracle.rel_l2(y, oracle.fft64(x, inverse=inv)) <= TOL_REL_L2


def test_three_pass_first_pass_unaligned_input(oracle, lib_built):
    """The device entry takes any 8-byte aligned input.  For N = 2^25 (three
    passes, the 8-column first pass, whose 16-byte stores go to the plan's
    workspace) an input one sample past a 16-byte boundary gives the same bits
    as the aligned host path."""
    torch = pytest.importorskip("torch")
    import numpy as np

    import gbfft
    from gbfft import signals
    n = 1 << 25
    x = signals.normal_c64(1, n, seed=1400)
    buf = torch.empty(n + 1, dtype=torch.complex64, device="cuda")
    buf[1:] = torch.from_numpy(x[0]).cuda()
    dx = buf[1:]
    assert dx.data_ptr() % 16 == 8
    dy = torch.empty(n, dtype=torch.complex64, device="cuda")
    with gbfft.Context(0) as ctx:
        for d in (gbfft.FORWARD, gbfft.INVERSE):
            aligned = ctx.c2c_host(x, d)
            ctx.c2c_device(dx, dy, n, 1, d)
            torch.cuda.synchronize()
            assert np.array_equal(dy.cpu().numpy()[None], aligned)


@pytest.mark.parametrize("logn,batch,loge", [(21, 3, 4), (22, 2, 4), (25, 1, 5)])
def test_three_pass_persistent_first_pass(tmp_path, monkeypatch, oracle, lib_built, logn, batch, loge):
    """Three-pass plans whose lone first pass runs as a persistent tile loop
    (L2 prefetch of the next tile), the last two passes fused: FP64 gate in
    both directions."""
    import numpy as np

    import gbfft
    from gbfft import signals
    cache = tmp_path / "tune.jsonl"
    lines = []
    for d in (gbfft.FORWARD, gbfft.INVERSE):
        line = json.loads(_cache_line(logn, batch, d, 10, 1, loge=loge))
        line["fused"] = 1
        lines.append(json.dumps(line))
    cache.write_text("\n".join(lines) + "\n")
    monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
    x = signals.normal_c64(batch, 1 << logn, seed=1000 + logn)
    with gbfft.Context(0) as ctx:
        y = ctx.c2c_host(x, gbfft.FORWARD)
        z = ctx.c2c_host(y, gbfft.INVERSE)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    assert oracle.rel_l2(y, ref) <= TOL_REL_L2
    assert oracle.rel_l2(z, x) <= 1e-6


@pytest.mark.parametrize("prec,tol", [(1, 2e-6), (3, 2e-6), (4, 2e-6)])
def test_autotune_split_form(tmp_path, monkeypatch, oracle, lib_built, prec, tol):
    """The tuner at a split precision times the split form's own candidates
    (fused pass pair, one launch per pass), caches the choice under that
    precision, and the chosen plan meets the form's FP64 gate."""
    import gbfft
    from gbfft import signals
    cache = tmp_path / "tune.jsonl"
    monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
    n, batch = 1 << 16, 8
    x = signals.tones_c64(batch, n, seed=77)
    with gbfft.Context(0) as ctx:
        ctx.set_precision(prec)
        assert ctx.autotune(n, batch, gbfft.FORWARD) > 0
        y = ctx.c2c_host(x, gbfft.FORWARD)
    assert oracle.rel_l2(y, oracle.fft64(x)) <= tol
    lines = [json.loads(l) for l in cache.read_text().splitlines()]
    assert len(lines) == 1 and lines[0]["precision"] == prec and lines[0]["logn"] == 16


@pytest.mark.parametrize("logn,batch", [(6, 40), (8, 37), (10, 9), (12, 5), (13, 3), (14, 2)])
def test_packed_and_scalar_butterflies_same_bits(tmp_path, monkeypatch, oracle, lib_built, logn, batch):
    """The single-pass kernel runs its butterflies and twiddles with packed
    two-lane FP32 instructions from N = 2^8, the persistent tile loop with
    scalar ones; each lane of a packed add, subtract, FMA or multiply rounds
    like the scalar operation, so both give the same bits in both directions
    (and meet the FP64 gate)."""
    import numpy as np

    import gbfft
    from gbfft import signals
    x = signals.normal_c64(batch, 1 << logn, seed=1400 + logn)
    outs = {}
    for persistent in (0, 1):
        cache = tmp_path / f"tune_p{persistent}.jsonl"
        cache.write_text("\n".join(_cache_line(logn, batch, d, 10, persistent, loge=4)
                                   for d in (gbfft.FORWARD, gbfft.INVERSE)) + "\n")
        monkeypatch.setenv("GBFFT_AUTOTUNE_CACHE", str(cache))
        with gbfft.Context(0) as ctx:
            outs[persistent] = [ctx.c2c_host(x, d) for d in (gbfft.FORWARD, gbfft.INVERSE)]
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    for y, inv in zip(outs[0], (False, True)):
        assert oracle.rel_l2(y, oracle.fft64(x, inverse=inv)) <= TOL_REL_L2
