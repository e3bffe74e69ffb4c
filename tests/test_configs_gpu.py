"""GPU parity at the benchmark configurations' own sizes and seeded inputs.

Each test runs one configuration exactly as the bench runs it (size, batch,
distribution, seed, default plan) through the C ABI and meets the oracles
on those same inputs:

  C2  N = 4096 x 16384, re/im iid N(0,1), seed 2: the WHOLE batch against
      the reference's Stockham path (oracle.ref_fft, max |a - b| <= 1e-3,
      src/benchmark.rs:45, 272-297) and against FP64 (rel-L2 <= 2e-6), both
      directions.
  C3  N = 2^26 x 1 and N = 2^22 x 64, N(0,1), seed 3, default (three-pass)
      plan: whole transforms against FP64 (rel-L2 <= 2e-6), both directions.
      The reference path is no gate here: its f32 twiddle angles put it more
      than 1e-3 from FP64 on its own benchmark input above N = 2^20.
  C4  N = 2^16 x 4096 tones workload in the split tensor-core forms: sampled
      rows against FP64 (2e-6 for FP16 and TF32 hi+lo and BF16 x 6, the FP32
      form's own budget), with the FP32 form on the same rows beside it.
  C5  the seeded 10,000-transform ragged set (one persistent launch): up to
      64 transforms of every (size, direction) against the reference path
      (1e-3) and FP64 (2e-6).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_REF = 1e-3     # the reference's VALIDATION_TOLERANCE, max |a - b| per complex sample
TOL_REL_L2 = 2e-6  # FP32 and split forms against FP64


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    assert t.cuda.is_available()
    return t


def _maxabs(a, b):
    return float(np.max(np.abs(np.asarray(a, np.complex128) - np.asarray(b, np.complex128))))


def test_c2_whole_batch_vs_reference_path_and_fp64(gpu_ctx, oracle, torch):
    import gbfft
    from gbfft import signals
    n, batch = 4096, 16384
    x = signals.normal_c64_torch(batch, n, seed=2)
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    s = torch.cuda.current_stream().cuda_stream
    gpu_ctx.c2c_device(x, y, n, batch, gbfft.FORWARD, stream=s)
    gpu_ctx.c2c_device(x, z, n, batch, gbfft.INVERSE, stream=s)
    torch.cuda.synchronize()
    xh = x.cpu().numpy()
    for out, inv in ((y, False), (z, True)):
        got = out.cpu().numpy()
        assert _maxabs(got, oracle.ref_fft(xh, inverse=inv, threads=16)) <= TOL_REF, inv
        assert oracle.rel_l2(got, oracle.fft64(xh, inverse=inv)) <= TOL_REL_L2, inv


@pytest.mark.parametrize("logn,batch,inv_rows", [(26, 1, 1), (22, 64, 16)])
def test_c3_default_plan_vs_fp64(gpu_ctx, oracle, torch, logn, batch, inv_rows):
    """The default plan of N = 2^26 (radix-2^10 first pass, then passes 2-3
    fused) and of N = 2^22 (radix-2^6 first pass, then the fused pair)."""
    import gbfft
    from gbfft import signals
    n = 1 << logn
    x = signals.normal_c64_torch(batch, n, seed=3)
    y = torch.empty_like(x)
    s = torch.cuda.current_stream().cuda_stream
    gpu_ctx.c2c_device(x, y, n, batch, gbfft.FORWARD, stream=s)
    torch.cuda.synchronize()
    xh = x.cpu().numpy()
    err = oracle.rel_l2(y.cpu().numpy(), oracle.fft64(xh))
    assert err <= TOL_REL_L2, err
    del y
    xi = x[:inv_rows].contiguous()
    z = torch.empty_like(xi)
    gpu_ctx.c2c_device(xi, z, n, inv_rows, gbfft.INVERSE, stream=s)
    torch.cuda.synchronize()
    err = oracle.rel_l2(z.cpu().numpy(), oracle.fft64(xh[:inv_rows], inverse=True))
    assert err <= TOL_REL_L2, err


@pytest.mark.parametrize("prec,tol", [(1, 2e-6), (3, 2e-6), (4, 2e-6)])
def test_c4_full_size_split_forms_vs_fp64(lib_built, oracle, torch, prec, tol):
    """N = 2^16 x 4096 (2^28 samples) in FP16 hi+lo (prec 1), TF32 hi+lo
    (prec 3) and BF16 x 6 (prec 4): 64 rows spread over the batch against
    FP64, forward and inverse, with the FP32 form on the same rows (both
    within the budget)."""
    import gbfft
    from gbfft import signals
    n, batch = 1 << 16, 4096
    rows = np.linspace(0, batch - 1, 64).astype(np.int64)
    with gbfft.Context(0) as ctx:
        x = signals.tones_c64_torch(batch, n, seed=4, ctx=ctx)
        y = torch.empty_like(x)
        s = torch.cuda.current_stream().cuda_stream
        xs = x[torch.from_numpy(rows).cuda()].cpu().numpy()
        for direction, inv in ((gbfft.FORWARD, False), (gbfft.INVERSE, True)):
            ref = oracle.fft64(xs, inverse=inv)
            errs = {}
            for p in (prec, gbfft.PREC_FP32):
                ctx.set_precision(p)
                ctx.c2c_device(x, y, n, batch, direction, stream=s)
                torch.cuda.synchronize()
                errs[p] = oracle.rel_l2(y[torch.from_numpy(rows).cuda()].cpu().numpy(), ref)
            assert errs[prec] <= tol, (inv, errs)
            assert errs[gbfft.PREC_FP32] <= TOL_REL_L2, (inv, errs)


def test_c5_seeded_set_vs_reference_path_and_fp64(gpu_ctx, oracle, torch):
    """The 10,000-transform set of the ragged workload, one persistent launch.
    Per (size, direction), the first 64 transforms in descriptor order meet
    FP64 at 2e-6 and the reference path at 1e-3.

    At N = 2^18 on these inputs (|X_k| up to ~1.5e3) the reference path itself
    is up to ~1.1e-3 from the exact transform, through its f32 twiddle angles
    (src/lib.rs:764-769).  A transform whose reference-path output is farther
    than 0.9e-3 from FP64 therefore cannot meet 1e-3 against it whatever this
    library computes; for those the test requires instead that this library
    is at most half as far from FP64 as the reference path is (so the miss is
    the reference path's own error), and that they are at most 5 % of the
    transforms checked."""
    import gbfft
    from gbfft import signals
    descs, total = signals.ragged_set(10000, seed=5)
    x = signals.uniform_c64_torch(1, total, seed=5)[0]
    y = torch.empty_like(x)
    plan = gpu_ctx.ragged_plan(descs)
    plan.execute(x, y, total, use_graph=True)
    plan.wait()
    xh = x.cpu().numpy()
    yh = y.cpu().numpy()
    groups = {}
    for off, L, d in descs.tolist():
        g = groups.setdefault((L, d), [])
        if len(g) < 64:
            g.append(off)
    checked, ref_over = 0, 0
    for (L, d), offs in sorted(groups.items()):
        n = 1 << L
        inv = d == gbfft.INVERSE
        xs = np.stack([xh[o:o + n] for o in offs])
        got = np.stack([yh[o:o + n] for o in offs])
        ref = oracle.ref_fft(xs, inverse=inv, threads=16)
        f64 = oracle.fft64(xs, inverse=inv)
        for i in range(len(offs)):
            checked += 1
            assert oracle.rel_l2(got[i], f64[i]) <= TOL_REL_L2, (L, d, i)
            d_ref = _maxabs(got[i], ref[i])
            if d_ref <= TOL_REF:
                continue
            ref_err = _maxabs(ref[i], f64[i])
            assert ref_err > 0.9 * TOL_REF, (L, d, i, d_ref, ref_err)
            assert _maxabs(got[i], f64[i]) <= 0.5 * ref_err, (L, d, i, ref_err)
            ref_over += 1
    assert checked == sum(len(v) for v in groups.values()) and len(groups) == 22
    assert ref_over <= 0.05 * checked, ref_over
    plan.close()
