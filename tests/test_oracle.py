"""CPU: pin the oracle against the reference's own known-answer tests and the
committed golden fixtures.  No GPU needed.

The reference's tests (larsjoost/wgls-rs-fft) compare GpuFft with rustfft
6.4.1 or with closed-form identities; rustfft is not in this environment, so
its role is taken by the FP64 oracle (validated against a direct DFT and
numpy's pocketfft), which is stricter.
"""
import numpy as np
import pytest

from conftest import golden

TOL = 1e-3  # src/benchmark.rs:45, tests/gpu_fft_test.rs:6


def maxdiff(a, b):
    return float(np.max(np.abs(np.asarray(a, np.complex128) - np.asarray(b, np.complex128))))


# ---- src/lib.rs:170-204: exact host-side helpers ---------------------------

def test_prepare_input_fft(oracle):
    x = np.array([1 + 2j, 3 + 4j], dtype=np.complex64)
    assert oracle.ref_prepare_input(x, False).tolist() == [1.0, 2.0, 3.0, 4.0]


def test_prepare_input_ifft(oracle):
    x = np.array([1 + 2j, 3 + 4j], dtype=np.complex64)
    assert oracle.ref_prepare_input(x, True).tolist() == [1.0, -2.0, 3.0, -4.0]


def test_inverse_postprocessing(oracle):
    y = oracle.ref_inverse_post(np.array([2 + 4j, 6 + 8j], dtype=np.complex64), 2)
    assert (y.real.tolist(), y.imag.tolist()) == ([1.0, 3.0], [-2.0, -4.0])


# ---- src/lib.rs:207-227: roundtrip of x_i = 0.1 i at N = 1024 (< 1e-4) ------

def test_roundtrip_consistency(oracle):
    x = golden("ref_signals.npz")["ramp"]
    y = oracle.ref_fft(oracle.ref_fft(x), inverse=True)[0]
    assert np.max(np.abs(y - x)) < 1e-4


# ---- tests/gpu_fft_test.rs and tests/ifft_test.rs (N = 1024, < 1e-3) -------

def test_fft_matches_fp64(oracle):
    g = golden("ref_signals.npz")
    out = oracle.ref_fft(g["rustfft_sig"])[0]
    assert maxdiff(out, g["rustfft_sig_f64"]) < TOL


def test_ifft_matches_fp64_roundtrip(oracle):
    x = golden("ref_signals.npz")["rustfft_sig"]
    spec = oracle.ref_fft(x)
    ours = oracle.ref_fft(spec, inverse=True)[0]
    ref = oracle.fft64(oracle.fft64(x), inverse=True)[0]
    assert maxdiff(ours, ref) < TOL


def test_fft_ifft_properties(oracle):
    x = golden("ref_signals.npz")["rustfft_sig"]
    spec = oracle.ref_fft(x)
    rec = oracle.ref_fft(spec, inverse=True)
    assert maxdiff(rec[0], x) < TOL
    spec2 = oracle.ref_fft(rec)
    assert maxdiff(spec2, spec) < TOL


# ---- tests/windowed_fft_test.rs (N = 2048 Hann window) ---------------------

def test_windowed_roundtrip(oracle):
    x = golden("ref_signals.npz")["hann2048"]
    rec = oracle.ref_fft(oracle.ref_fft(x), inverse=True)[0]
    assert maxdiff(rec, x) < TOL


def test_window_power_ratio_and_peaks(oracle):
    g = golden("ref_signals.npz")
    w = oracle.ref_fft(g["hann2048"])[0]
    o = oracle.ref_fft(g["tone2048"])[0]
    ratio = np.sum(np.abs(w) ** 2) / np.sum(np.abs(o) ** 2)
    assert 0.1 < ratio < 10.0
    p = np.abs(w) ** 2
    peaks = [i for i in range(1, 1024) if p[i] > p[i - 1] and p[i] > p[i + 1] and p[i] > 10.0]
    assert 10 in peaks and 50 in peaks


# ---- examples/test_parallel.rs, examples/compare_cufft.rs ------------------

def test_impulse_flat_spectrum(oracle):
    x = golden("ref_signals.npz")["impulse256"]
    out = oracle.ref_fft(x)[0]
    assert np.all(np.abs(np.abs(out) - 1.0) < 1e-3)


def test_batch_results_independent(oracle):
    n = 128
    sig = np.array([[(i * 10 + j) * 0.001 for j in range(n)] for i in range(4)], dtype=np.float32).astype(np.complex64)
    batch = oracle.ref_fft(sig)
    for i in range(4):
        assert maxdiff(oracle.ref_fft(sig[i])[0], batch[i]) < 1e-4


# ---- the two restatements and the FP64 oracle agree ------------------------

@pytest.mark.parametrize("logn", list(range(0, 13)))
def test_c_restatement_equals_numpy_restatement(oracle, logn):
    x = golden("sweep.npz")[f"x{logn}"]
    for inv in (False, True):
        assert np.array_equal(oracle.ref_fft(x, inv), oracle.ref_fft_numpy(x, inv))


@pytest.mark.parametrize("logn", list(range(0, 11)))
def test_fft64_equals_direct_dft(oracle, logn):
    x = golden("sweep.npz")[f"x{logn}"][0].astype(np.complex128)
    for inv in (False, True):
        a = oracle.fft64(x, inv)[0]
        b = oracle.dft64(x, inv)
        assert oracle.rel_l2(a, b) < 1e-13


@pytest.mark.parametrize("logn", [0, 1, 5, 12, 16, 20])
def test_fft64_equals_numpy(oracle, logn):
    from gbfft import signals
    x = signals.uniform_c64(2, 1 << logn, seed=11)
    a = oracle.fft64(x)
    b = np.fft.fft(x.astype(np.complex128), axis=1)
    assert oracle.rel_l2(a, b) < 1e-13


def test_reference_path_within_tolerance_of_fp64(oracle):
    """The reference path itself passes its own 1e-3 gate against FP64."""
    g = golden("sweep.npz")
    for L in range(0, 13):
        assert maxdiff(g[f"ref_{L}"], g[f"f64_{L}"]) < TOL


def test_bad_size_rejected(oracle):
    with pytest.raises(ValueError, match="non-zero power of two"):
        oracle.ref_fft(np.zeros((1, 3), np.complex64))


# ---- fixtures re-derive bit-for-bit ----------------------------------------

def test_golden_c1_rederives(oracle):
    import make_golden
    g = golden("c1.npz")
    x = make_golden.c1_input()
    assert np.array_equal(x, g["x"])
    assert np.array_equal(oracle.ref_fft(x), g["ref_fwd"])
    assert np.array_equal(oracle.ref_fft(x, True), g["ref_inv"])
    assert np.allclose(oracle.fft64(x), g["f64_fwd"], rtol=0, atol=1e-12)
    assert np.allclose(oracle.fft64(x, True), g["f64_inv"], rtol=0, atol=1e-12)


def test_golden_sweep_rederives(oracle):
    from gbfft import signals
    g = golden("sweep.npz")
    for L in range(0, 13):
        x = signals.uniform_c64(3, 1 << L, seed=7)
        assert np.array_equal(x, g[f"x{L}"])
        assert np.array_equal(oracle.ref_fft(x), g[f"ref_{L}"])
