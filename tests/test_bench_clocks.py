"""CPU: bench.py's clock record.  Samples taken before the GPU was busy are
left out of the median, and when the timed region is too short for enough
samples, the sampler keeps the same steps running (outside the timed
region) until they arrive, or gives up after its time limit."""
import time

import bench


def _line(sm, smax=2070, reasons=("Not Active",) * 4):
    return f"0, {sm}, {smax}, 900.0, 0x0, {', '.join(reasons)}"


def test_summary_ignores_samples_before_busy():
    s = bench.ClockSampler(0)
    s.lines = [(1.0, _line(345)), (2.0, _line(2070)), (3.0, _line(2070)),
               (4.0, _line(1980, reasons=("Not Active", "Not Active", "Not Active", "Active")))]
    out = s.summary(1.5)
    assert out["samples"] == 3 and out["sm_mhz"] == 2070 and out["sm_max_mhz"] == 2070
    assert out["reasons"] == ["sw_power_cap"]
    assert s.summary(10.0)["sm_mhz"] is None


def test_keep_busy_runs_until_samples_or_deadline():
    class FakeProc:
        pass

    s = bench.ClockSampler(0)
    s.proc = FakeProc()
    t0 = time.time()
    calls = []

    def step():
        calls.append(1)
        if len(calls) % 4 == 0:  # one sample arrives per batch of steps
            s.lines.append((time.time(), _line(2070)))

    s.keep_busy(t0, step, lambda: None, want=3, max_s=5.0)
    assert s.count_since(t0) == 3 and len(calls) == 12
    s2 = bench.ClockSampler(0)
    s2.proc = FakeProc()
    t1 = time.time()
    s2.keep_busy(t1, lambda: None, lambda: None, want=3, max_s=0.05)  # nothing arrives: bounded
    assert time.time() - t1 < 2.0 and s2.count_since(t1) == 0
    s3 = bench.ClockSampler(0)  # no nvidia-smi: nothing to wait for
    s3.keep_busy(time.time(), lambda: (_ for _ in ()).throw(AssertionError("ran")), lambda: None)
