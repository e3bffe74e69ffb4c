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


def _cache_line(logn, batch, direction, max_logr, persistent, precision=0, tile=0):
    return json.dumps({"arch": "sm_103", "logn": logn, "precision": precision, "direction": direction,
                       "batch_log2": batch.bit_length() - 1, "max_logr": max_logr, "persistent": persistent,
                       "fused": 0, "tile": tile, "seconds": 1.0})


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
