"""CPU: seeded generators, and the C ABI library (loads, exports every symbol
include/gbfft.h declares, reports no device here).  No compute calls."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def test_pcg_matches_reference_formula():
    """examples/parallel_pipeline.rs:36-40 evaluated by hand in Python ints."""
    from gbfft import signals

    def pcg(v):
        s = (v * 747796405 + 2891336453) & 0xFFFFFFFF
        w = (((s >> ((s >> 28) + 4)) ^ s) * 277803737) & 0xFFFFFFFF
        return (w >> 22) ^ w

    vs = np.array([0, 1, 2, 12345, 0xFFFFFFFF, 0x80000000], dtype=np.uint32)
    assert signals.pcg_np(vs).tolist() == [pcg(int(v)) for v in vs]


def test_uniform_range_and_determinism():
    from gbfft import signals
    a = signals.uniform_c64(4, 1024, seed=1)
    b = signals.uniform_c64(4, 1024, seed=1)
    c = signals.uniform_c64(4, 1024, seed=2)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    f = a.view(np.float32)
    assert f.min() >= -1.0 and f.max() < 1.0
    assert abs(float(f.mean())) < 0.02


def test_normal_moments():
    from gbfft import signals
    x = signals.normal_c64(64, 4096, seed=2).view(np.float32).astype(np.float64)
    assert abs(x.mean()) < 0.01 and abs(x.std() - 1.0) < 0.01


def test_chunking_is_invisible():
    from gbfft import signals
    a = signals.uniform_c64(1, (1 << 24) + 77, seed=3)
    idx = np.array([0, 5, (1 << 24) - 1, 1 << 24, (1 << 24) + 76])
    b = signals.uniform_c64(1, 16, seed=3)
    assert np.array_equal(a[0, :16], b[0])
    assert np.isfinite(a[0, idx]).all()


def header_symbols():
    src = open(os.path.join(ROOT, "include", "gbfft.h")).read()
    return sorted(set(re.findall(r"\b(gbfft_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib_built):
    import gbfft
    L = gbfft.load()
    declared = header_symbols()
    assert len(declared) >= 12
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(gbfft.SIGNATURES), "binding and header disagree"


def test_version_and_status_strings(lib_built):
    import gbfft
    L = gbfft.load()
    assert b"sm_103a" in L.gbfft_version()
    # The reference's own error messages (src/lib.rs:508, 530).
    assert gbfft.status_string(gbfft.ERR_INVALID_SIZE) == "Transform length must be a non-zero power of two"
    assert gbfft.status_string(gbfft.ERR_LENGTH_MISMATCH) == "All input vectors in a batch must have the same length"


def _have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_have_gpu(), reason="checks the no-GPU behaviour")
def test_no_device_here(lib_built):
    import gbfft
    assert gbfft.is_available() is False
    with pytest.raises(gbfft.GbfftError) as ei:
        gbfft.Context(0)
    assert ei.value.status == gbfft.ERR_NO_DEVICE


def test_product_does_not_reference_oracle():
    """The product path never imports, links or loads the oracle."""
    pkg = os.path.join(ROOT, "wgls-rs-fft_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".cpp", ".hpp")):
                text = open(os.path.join(dirpath, f)).read()
                assert "liboracle" not in text and "import oracle" not in text, f


def test_every_environment_variable_is_documented():
    """Every GBFFT_* variable the library reads with getenv appears in the
    header's environment list."""
    csrc = os.path.join(ROOT, "wgls-rs-fft_gb300", "csrc")
    read = set()
    for f in os.listdir(csrc):
        if f.endswith((".cu", ".cuh", ".h")):
            read |= set(re.findall(r'getenv\("(GBFFT_[A-Z0-9_]+)"\)', open(os.path.join(csrc, f)).read()))
    header = open(os.path.join(ROOT, "include", "gbfft.h")).read()
    env_doc = header[header.index("Environment read by the library"):]
    assert read, "no getenv found"
    missing = sorted(v for v in read if not re.search(r"\b%s\b" % v, env_doc))
    assert not missing, missing
