"""GPU: ragged batches (mixed sizes and directions in one persistent launch)
through the C ABI, against the FP64 oracle and the uniform entry point.

Gates: relative L2 <= 2e-6 per transform against FP64; the uniform entry
point's result for the same transform to the same tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_REL_L2 = 2e-6


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    assert t.cuda.is_available()
    return t


def _mixed_descs(sizes, dirs, gap=3):
    """Descriptors with gaps between transforms (offsets not aligned to N)."""
    import gbfft
    out, off = [], 5
    for L, d in zip(sizes, dirs):
        out.append((off, L, d))
        off += (1 << L) + gap
    return gbfft.ragged_descs(out), off


def _check_each(oracle, x, y, descs):
    for off, L, d in descs.tolist():
        n = 1 << L
        ref = oracle.fft64(x[off:off + n][None, :], inverse=(d == 1))[0]
        err = oracle.rel_l2(y[off:off + n], ref)
        assert err <= TOL_REL_L2, (off, L, d, err)


def test_ragged_all_sizes_both_directions(gpu_ctx, oracle, torch):
    import gbfft
    from gbfft import signals
    rng = np.random.default_rng(7)
    sizes = list(range(0, 19)) * 2 + [int(v) for v in rng.integers(8, 19, size=30)]
    rng.shuffle(sizes)
    dirs = [int(v) for v in rng.choice([-1, 1], size=len(sizes))]
    descs, total = _mixed_descs(sizes, dirs)
    x = signals.uniform_c64(1, total, seed=41)[0]
    d_in = torch.from_numpy(x).cuda()
    d_out = torch.full_like(d_in, float("nan"))
    plan = gpu_ctx.ragged_plan(descs)
    plan.execute(d_in, d_out, total, use_graph=False)
    plan.wait()
    y = d_out.cpu().numpy()
    _check_each(oracle, x, y, descs)
    # same transforms through the uniform entry point
    for off, L, d in descs.tolist()[:12]:
        n = 1 << L
        want = gpu_ctx.c2c_host(x[off:off + n][None, :], d)[0]
        assert oracle.rel_l2(y[off:off + n], want) <= TOL_REL_L2
    # samples outside every transform are untouched
    mask = np.ones(total, bool)
    for off, L, _ in descs.tolist():
        mask[off:off + (1 << L)] = False
    assert np.isnan(y[mask]).all()
    plan.close()


def test_ragged_graph_replay_and_in_place(gpu_ctx, oracle, torch):
    from gbfft import signals
    descs, total = _mixed_descs([9, 15, 4, 18, 12, 14, 0], [-1, 1, 1, -1, -1, 1, -1])
    x = signals.normal_c64(1, total, seed=42)[0]
    d_in = torch.from_numpy(x).cuda()
    d_out = torch.zeros_like(d_in)
    plan = gpu_ctx.ragged_plan(descs)
    plan.execute(d_in, d_out, total, use_graph=True)
    plan.wait()
    y1 = d_out.cpu().numpy().copy()
    d_out.zero_()
    plan.execute(d_in, d_out, total, use_graph=True)  # replay
    plan.wait()
    assert np.array_equal(d_out.cpu().numpy(), y1)
    _check_each(oracle, x, y1, descs)
    d_io = d_in.clone()
    plan.execute(d_io, d_io, total, use_graph=True)  # new pointers: recaptured; in place
    plan.wait()
    _check_each(oracle, x, d_io.cpu().numpy(), descs)
    assert plan.launch_count() == 3
    plan.close()


def test_ragged_one_shot_and_errors(gpu_ctx, torch):
    import gbfft
    from gbfft import signals
    descs, total = _mixed_descs([10, 16], [-1, -1])
    x = signals.uniform_c64(1, total, seed=43)[0]
    d = torch.from_numpy(x).cuda()
    o = torch.empty_like(d)
    gpu_ctx.ragged_device(d, o, total, descs)
    extent = max(off + (1 << L) for off, L, _ in descs.tolist())
    gpu_ctx.ragged_device(d, o, extent, descs)
    with pytest.raises(gbfft.GbfftError) as e:
        gpu_ctx.ragged_device(d, o, extent - 1, descs)  # capacity check
    assert e.value.status == gbfft.ERR_INVALID_ARGUMENT
    with pytest.raises(gbfft.GbfftError) as e:
        gpu_ctx.ragged_plan([(0, 19, -1)])
    assert e.value.status == gbfft.ERR_UNSUPPORTED
    with pytest.raises(gbfft.GbfftError) as e:
        gpu_ctx.ragged_plan([(0, 8, 0)])
    assert e.value.status == gbfft.ERR_INVALID_ARGUMENT
    empty = gpu_ctx.ragged_plan([])
    empty.execute(0, 0, 0)
    empty.wait()
    empty.close()


def test_ragged_dependency_wait_times_out(gpu_ctx, torch):
    """Failure path: the first-pass items are dropped on the host, so the
    second-pass items wait on counters nothing increments; the bounded wait
    must give up, report GBFFT_ERR_TIMEOUT, and leave the context usable."""
    import gbfft
    from gbfft import signals
    descs, total = _mixed_descs([15, 16, 8], [-1, 1, -1])
    x = signals.uniform_c64(1, total, seed=44)[0]
    d = torch.from_numpy(x).cuda()
    o = torch.zeros_like(d)
    plan = gpu_ctx.ragged_plan(descs)
    plan.set(gbfft.RAGGED_OPT_SPIN_LIMIT, 2000)
    plan.set(gbfft.RAGGED_OPT_TEST_DROP_PRODUCERS, 1)
    plan.execute(d, o, total, use_graph=False)
    with pytest.raises(gbfft.GbfftError) as e:
        plan.wait()
    assert e.value.status == gbfft.ERR_TIMEOUT
    plan.set(gbfft.RAGGED_OPT_TEST_DROP_PRODUCERS, 0)
    plan.execute(d, o, total, use_graph=True)
    plan.wait()
    plan.close()
    y = gpu_ctx.c2c_host(x[:64][None, :], gbfft.FORWARD)  # context still healthy
    assert np.isfinite(y).all()


def test_ragged_full_workload_roundtrip(gpu_ctx, oracle, torch):
    """10,000 transforms, log2 N uniform on 8..18, directions 50/50 (~4 GB):
    sampled transforms against FP64 and the whole set through a second plan
    with every direction flipped (must give back the input)."""
    import gbfft
    from gbfft import signals
    descs, total = signals.ragged_set(10000, seed=5)
    x = signals.uniform_c64_torch(1, total, seed=5)[0]
    y = torch.empty_like(x)
    plan = gpu_ctx.ragged_plan(descs)
    plan.execute(x, y, total, use_graph=True)
    plan.wait()
    flipped = descs.copy()
    flipped["direction"] = -flipped["direction"]
    back = gpu_ctx.ragged_plan(flipped)
    z = torch.empty_like(x)
    back.execute(y, z, total, use_graph=True)
    back.wait()
    rt = (torch.linalg.vector_norm(z - x) / torch.linalg.vector_norm(x)).item()
    assert rt < 1e-6
    # one sampled transform of every size against FP64
    seen = set()
    for off, L, d in descs.tolist():
        if L in seen:
            continue
        seen.add(L)
        n = 1 << L
        xs = x[off:off + n].cpu().numpy()
        ref = oracle.fft64(xs[None, :], inverse=(d == 1))[0]
        assert oracle.rel_l2(y[off:off + n].cpu().numpy(), ref) <= TOL_REL_L2, (L, d)
    assert len(seen) == 11
    plan.close()
    back.close()


@pytest.mark.parametrize("prec,tol", [(1, 2e-6), (2, 2e-5), (3, 2e-6), (4, 2e-6)])
def test_ragged_split_tensor_core_form(lib_built, oracle, torch, prec, tol):
    """The ragged launch in the split tensor-core forms (the context's
    precision when the plan is made): two-pass transforms (N = 2^14..2^18) run
    their radix-16 butterflies on tcgen05, single-pass ones stay FP32.  Gates
    as for the uniform split form: FP16 and TF32 hi+lo at rel-L2 <= 2e-6
    against FP64, BF16x3 at 2e-5; graph replay repeats the result exactly; in place works."""
    import gbfft
    from gbfft import signals
    rng = np.random.default_rng(8)
    sizes = list(range(8, 19)) + [int(v) for v in rng.integers(12, 19, size=20)]
    dirs = [int(v) for v in rng.choice([-1, 1], size=len(sizes))]
    descs, total = _mixed_descs(sizes, dirs)
    x = signals.uniform_c64(1, total, seed=45)[0]
    with gbfft.Context(0) as ctx:
        ctx.set_precision(prec)
        d_in = torch.from_numpy(x).cuda()
        d_out = torch.full_like(d_in, float("nan"))
        plan = ctx.ragged_plan(descs)
        plan.execute(d_in, d_out, total, use_graph=True)
        plan.wait()
        y = d_out.cpu().numpy()
        for off, L, d in descs.tolist():
            n = 1 << L
            ref = oracle.fft64(x[off:off + n][None, :], inverse=(d == 1))[0]
            assert oracle.rel_l2(y[off:off + n], ref) <= tol, (L, d)
        plan.execute(d_in, d_out, total, use_graph=True)
        plan.wait()
        assert np.array_equal(d_out.cpu().numpy(), y, equal_nan=True)  # gaps stay NaN
        d_io = d_in.clone()
        plan.execute(d_io, d_io, total, use_graph=False)
        plan.wait()
        assert np.array_equal(d_io.cpu().numpy()[~np.isnan(y)], y[~np.isnan(y)])
        plan.close()


def test_ragged_split_form_wait_times_out(lib_built, torch):
    """The dropped-producer failure path in the tensor-core ragged kernel: the
    bounded dependency wait gives up, GBFFT_ERR_TIMEOUT is reported, TMEM is
    released and the context keeps working."""
    import gbfft
    from gbfft import signals
    descs, total = _mixed_descs([15, 17, 9], [-1, 1, -1])
    x = signals.uniform_c64(1, total, seed=46)[0]
    with gbfft.Context(0) as ctx:
        ctx.set_precision(gbfft.PREC_TC_FP16)
        d = torch.from_numpy(x).cuda()
        o = torch.zeros_like(d)
        plan = ctx.ragged_plan(descs)
        plan.set(gbfft.RAGGED_OPT_SPIN_LIMIT, 2000)
        plan.set(gbfft.RAGGED_OPT_TEST_DROP_PRODUCERS, 1)
        plan.execute(d, o, total, use_graph=False)
        with pytest.raises(gbfft.GbfftError) as e:
            plan.wait()
        assert e.value.status == gbfft.ERR_TIMEOUT
        plan.set(gbfft.RAGGED_OPT_TEST_DROP_PRODUCERS, 0)
        plan.execute(d, o, total, use_graph=False)
        plan.wait()
        plan.close()
        ctx.set_precision(gbfft.PREC_FP32)
        assert np.isfinite(ctx.c2c_host(x[:256][None, :], gbfft.FORWARD)).all()


def test_ragged_lag_option(lib_built, torch):
    """GBFFT_RAGGED_OPT_LAG only reorders the work queue: every lag gives the
    same bits; values outside 1..64 are refused."""
    import gbfft
    from gbfft import signals
    descs, total = _mixed_descs([16, 18, 10, 17, 12, 15], [-1, 1, 1, -1, -1, 1])
    x = signals.uniform_c64(1, total, seed=47)[0]
    with gbfft.Context(0) as ctx:
        d = torch.from_numpy(x).cuda()
        outs = []
        plan = ctx.ragged_plan(descs)
        for lag in (4, 1, 16):
            plan.set(gbfft.RAGGED_OPT_LAG, lag)
            o = torch.full_like(d, float("nan"))
            plan.execute(d, o, total, use_graph=True)
            plan.wait()
            outs.append(o.cpu().numpy())
        for v in (0, 65):
            with pytest.raises(gbfft.GbfftError) as e:
                plan.set(gbfft.RAGGED_OPT_LAG, v)
            assert e.value.status == gbfft.ERR_INVALID_ARGUMENT
        plan.close()
    assert np.array_equal(outs[0], outs[1], equal_nan=True) and np.array_equal(outs[0], outs[2], equal_nan=True)
