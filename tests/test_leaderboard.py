"""The rivalry leaderboard (gbfft.leaderboard), mirroring the reference's
examples/rivalry_leaderboard.rs: its batch rule and tests (:147-202), its
benchmark input (src/benchmark.rs:112-122), table and validation at 1e-3;
the GPU test runs the registered rivals."""
import numpy as np
import pytest


def test_choose_batch_size_matches_reference_rule(lib_built):
    from gbfft import leaderboard as lb
    assert lb.choose_batch_size(256) == 1024 and lb.choose_batch_size(1024) == 1024
    assert lb.choose_batch_size(16384) == 256 and lb.choose_batch_size(65536) == 64
    assert lb.choose_batch_size(262_144) == 16 and lb.choose_batch_size(1_048_576) == 1
    for n in (1, 2, 256, 1024, 16384, 65536, 262_144, 1_048_576, 1 << 26):
        b = lb.choose_batch_size(n)
        assert b >= 1 and (n * b <= lb.MAX_TOTAL_SAMPLES or b == 1)


def test_pipeline_input_and_validation(lib_built):
    from gbfft import leaderboard as lb
    rows = lb.pipeline_input(8, 2)
    t = np.arange(8, dtype=np.float32) / np.float32(8)
    assert rows[0].dtype == np.complex64 and len(rows) == 2
    assert np.allclose(rows[1].real, t * 0.001) and np.allclose(rows[1].imag, np.sin(2 * np.pi * t) * 0.001)
    ref = lb.baseline_fft(rows)
    assert lb.validate([r.astype(np.complex64) for r in ref], ref) is None
    bad = [ref[0] + 2e-3, ref[1]]
    assert lb.validate(bad, ref) == pytest.approx(2e-3, rel=1e-6)


def test_run_rival_and_table_with_a_cpu_rival(lib_built):
    from gbfft import leaderboard as lb
    from gbfft.gpu_fft import FftExecutor

    class NumpyRival(FftExecutor):
        def name(self):
            return "numpy f32"

        def fft(self, inputs):
            return list(np.fft.fft(np.stack(inputs), axis=1).astype(np.complex64))

    ticks = iter([0.0, 0.5])
    r = lb.run_rival(NumpyRival(), 256, 4, clock=lambda: next(ticks))
    assert r.status == "PASS" and r.batch == 4
    assert r.msamples_per_sec == pytest.approx(256 * 4 / 0.05 / 1e6)
    assert r.gflops == pytest.approx(5 * 256 * 4 * 8 / 0.05 / 1e9)
    table = lb.format_table(256, [r, lb.Result("broken", 4, None, None, "UNSUPPORTED")])
    assert "--- N = 256 ---" in table and "numpy f32" in table and "ERROR" in table and "UNSUPPORTED" in table


@pytest.mark.gpu
def test_leaderboard_rivals_pass_on_gpu(lib_built, capsys):
    import gbfft
    from gbfft import leaderboard as lb
    rivals = lb.default_rivals()
    names = [r.name() for r in rivals]
    assert any("GB300" in n for n in names) and any("cuFFT" in n for n in names)
    for n in (1024, 65536):
        results = [lb.run_rival(r, n, lb.choose_batch_size(n)) for r in rivals]
        for res in results:
            assert res.status == "PASS", (n, res)
            assert res.msamples_per_sec > 0
    assert lb.main(["--sizes", "256"]) == 0
    assert "RIVALRY LEADERBOARD" in capsys.readouterr().out


NCU_CSV = '''==PROF== Connected to process 1
"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size","Grid Size","Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"
"0","7","python3.12","h","void gbfft::fft_rows_kernel<10, 11>(const float2 *, float2 *)","1","7","(128, 1, 1)","(512, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_read.sum","byte","8,388,608"
"0","7","python3.12","h","void gbfft::fft_rows_kernel<10, 11>(const float2 *, float2 *)","1","7","(128, 1, 1)","(512, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_write.sum","byte","8388608"
"0","7","python3.12","h","void gbfft::fft_rows_kernel<10, 11>(const float2 *, float2 *)","1","7","(128, 1, 1)","(512, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","ns","4000"
"1","7","python3.12","h","void gbfft::fft_rows_kernel<10, 11>(const float2 *, float2 *)","1","7","(128, 1, 1)","(512, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_read.sum","byte","8388608"
"1","7","python3.12","h","void gbfft::fft_rows_kernel<10, 11>(const float2 *, float2 *)","1","7","(128, 1, 1)","(512, 1, 1)","0","10.3","Command line profiler metrics","dram__bytes_write.sum","byte","8388608"
"1","7","python3.12","h","void gbfft::fft_rows_kernel<10, 11>(const float2 *, float2 *)","1","7","(128, 1, 1)","(512, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","us","6"
"2","7","python3.12","h","void gbfft::twiddle_fill_kernel(float2 *)","1","7","(256, 1, 1)","(4, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","ns","1500"
"3","7","python3.12","h","void fft_rows_kernel<12, 12, (int)-1, 4>(const float2 *, float2 *)","1","7","(256, 1, 1)","(8, 1, 1)","0","10.3","Command line profiler metrics","gpu__time_duration.sum","ns","900"
'''


def test_parse_ncu_csv_aggregates_per_kernel(lib_built):
    from gbfft import leaderboard as lb
    ks = lb.parse_ncu_csv(NCU_CSV)
    assert [k.kernel for k in ks] == ["gbfft::fft_rows_kernel<10, 11>", "gbfft::twiddle_fill_kernel",
                                      "fft_rows_kernel<12, 12, (int)-1, 4>"]
    rows = ks[0]
    assert rows.launches == 2 and rows.seconds == pytest.approx(10e-6) and rows.dram_bytes == 4 * 8388608
    assert ks[1].launches == 1 and ks[1].dram_bytes == 0
    assert lb.parse_ncu_csv("no csv here") == []
    text = lb.format_counters(1024, 1024, "GB300 FP32", ks)
    assert "4 launch(es)" in text and "fft_rows_kernel" in text


def test_ncu_counters_runs_plain_first_then_ncu(lib_built, tmp_path):
    """The captures run only after the same child command exited 0 without
    ncu; a failing plain run raises before ncu is started.  The first capture
    is a launch list with device time only; DRAM counters are then collected
    for the dominant kernel alone, one launch."""
    from gbfft import leaderboard as lb
    calls = []

    class R:
        def __init__(self, rc):
            self.returncode, self.stderr, self.stdout = rc, "", ""

    def fake_run(cmd, **kw):
        calls.append(cmd)
        if cmd[0] == "ncu":
            log = cmd[cmd.index("--log-file") + 1]
            with open(log, "w") as f:
                f.write(NCU_CSV)
            assert "--clock-control" in cmd and cmd[cmd.index("--clock-control") + 1] == "none"
        return R(0)

    ks = lb.ncu_counters(1024, 0, run=fake_run)
    assert len(calls) == 3 and calls[0][0] != "ncu" and calls[1][0] == "ncu" and calls[2][0] == "ncu"
    assert calls[1][calls[1].index("--metrics") + 1] == "gpu__time_duration.sum"
    assert "-k" not in calls[1] and "-c" not in calls[1]
    assert calls[2][calls[2].index("--metrics") + 1] == "dram__bytes_read.sum,dram__bytes_write.sum"
    assert calls[2][calls[2].index("-k") + 1] == "regex:fft_rows_kernel" and calls[2][calls[2].index("-c") + 1] == "1"
    assert ks[0].launches == 2 and ks[0].dram_bytes == 4 * 8388608  # two launches of 2 x 8 MB (fake data)
    assert ks[1].dram_bytes != ks[1].dram_bytes  # nan: not captured
    with pytest.raises(RuntimeError):
        lb.ncu_counters(1024, 0, run=lambda cmd, **kw: R(1))
