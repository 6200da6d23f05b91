"""Host-side pieces of bench.py: the DRAM traffic and the executed instructions of the
dominant kernel come from committed ncu captures (profiles/kernel_counters.json) and are
reported only for the workload and batch they were captured at; every capture command
keeps the GPU clocks as they are (--clock-control none); the FP64 roof comes from the
committed DGEMM measurement."""

import importlib.util
import json
import os

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(REPO, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _counters():
    with open(os.path.join(REPO, "profiles", "kernel_counters.json")) as f:
        return json.load(f)


def test_counter_records_are_well_formed():
    rec = _counters()
    assert rec, "no captures"
    for workload, r in rec.items():
        assert workload in _bench().WORKLOADS
        assert r["dram_bytes_per_launch"] == r["dram_bytes_read_per_launch"] + r["dram_bytes_write_per_launch"]
        assert r["dram_bytes_per_launch"] > 0 and r["batch"] > 0 and r["launches"] > 0
        if "warp_instructions_per_launch" in r:
            assert r["warp_instructions_per_launch"] > 0
        assert "--clock-control none" in r["command"] and r["command"].startswith("ncu ")


def test_counters_only_for_the_captured_workload_and_batch():
    b = _bench()
    for workload, r in _counters().items():
        assert b.captured_traffic(workload, r["batch"]) == r["dram_bytes_per_launch"]
        assert b.captured_traffic(workload, r["batch"] + 1) is None
    assert b.captured_traffic("no_such_workload", 512) is None


def test_fp64_peak_record():
    b = _bench()
    tf, src = b.fp64_peak()
    assert 0.1 < tf < 100.0 and "profiles/fp64_peak.json" in src
    with open(os.path.join(REPO, "profiles", "fp64_peak.json")) as f:
        rec = json.load(f)
    assert rec["command"] and rec["gpu_name"]


def test_cpu_model_is_named():
    assert _bench().cpu_model()
