"""Host-side pieces of bench.py: the DRAM traffic of the dominant kernel comes from the
committed one-pass ncu capture (profiles/dram_traffic.json) and is reported only for the
workload and batch it was captured at; every capture command keeps the GPU clocks as
they are (--clock-control none)."""

import importlib.util
import json
import os

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(REPO, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_records_are_well_formed():
    with open(os.path.join(REPO, "profiles", "dram_traffic.json")) as f:
        rec = json.load(f)
    assert rec, "no captures"
    for workload, r in rec.items():
        assert workload in _bench().WORKLOADS
        assert r["dram_bytes_per_launch"] == r["dram_bytes_read_per_launch"] + r["dram_bytes_write_per_launch"]
        assert r["dram_bytes_per_launch"] > 0 and r["batch"] > 0 and r["launches"] > 0
        assert "--clock-control none" in r["command"] and r["command"].startswith("ncu ")


def test_traffic_only_for_the_captured_workload_and_batch():
    b = _bench()
    with open(os.path.join(REPO, "profiles", "dram_traffic.json")) as f:
        rec = json.load(f)
    for workload, r in rec.items():
        assert b.captured_traffic(workload, r["batch"]) == r["dram_bytes_per_launch"]
        assert b.captured_traffic(workload, r["batch"] + 1) is None
    assert b.captured_traffic("no_such_workload", 512) is None
