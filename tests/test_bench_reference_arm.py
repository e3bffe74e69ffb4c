"""CPU: `bench.py --impl reference`, the reference arm.  It times the reference's
own CPU path for the hot path (the Stockham R4/R2 f32 restatement in C, all
host threads) on a bounded sample of the workload and prints one JSON line
with the bench contract's keys; under torchrun only rank 0 works and prints.
No GPU is involved."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT

BENCH = os.path.join(ROOT, "bench.py")


def _lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _run(*extra, timeout=600):
    r = subprocess.run([sys.executable, BENCH, "--impl", "reference", "--steps", "3", "--warmup", "3", *extra],
                       capture_output=True, text=True, timeout=timeout, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1, r.stdout
    return lines[0]


def _check_contract(line):
    sys.path.insert(0, ROOT)
    import bench
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 3 and line["warmup"] == 3 and line["ms_per_step"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["unit"] == line["unit"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert line["gpu_launches"] == 0


def test_reference_arm_default_workload():
    line = _run()
    _check_contract(line)
    assert line["config"]["workload"] == "n4096_b16384"
    assert "N(0,1)" in line["data"]


def test_reference_arm_uniform_and_ragged_workloads():
    line = _run("--workload", "n1024_b9")
    _check_contract(line)
    assert line["config"]["n"] == 1024 and "U[-1,1)" in line["data"]
    line = _run("--workload", "ragged_c5", "--ragged-count", "300")
    _check_contract(line)
    assert line["config"]["workload"] == "ragged_c5" and line["config"]["transforms"] == 300
    assert "transforms" in line["cpu_baseline"]["sample"]
    line = _run("--workload", "pipeline_n1024_b8")
    _check_contract(line)
    assert line["config"]["n"] == 1024 and line["config"]["batch"] == 8 and "window" in line["cpu_baseline"]["sample"]


def test_reference_arm_under_torchrun_prints_once():
    """Two ranks on 127.0.0.1: rank 0 times and prints, rank 1 exits 0 without work."""
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", str(port), BENCH, "--impl", "reference",
                        "--gpus", "2", "--steps", "3", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1, r.stdout
    _check_contract(lines[0])
    assert lines[0]["n_gpus"] == 2
