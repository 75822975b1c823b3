"""Host-side pieces of bench.py that need no GPU: the DRAM traffic figure of the
roofline comes from the committed ncu summary only for the workload that
summary was captured on."""

import importlib.util
import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_only_for_the_captured_workload():
    b = _bench()
    with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
        summary = json.load(f)
    key = summary["workload_key"]
    for kernel, entry in summary["kernels"].items():
        assert b._ncu_traffic(kernel, key) == entry["bytes_per_launch"]
        assert entry["bytes_per_launch"] == entry["read_bytes"] + entry["write_bytes"]
        assert b._ncu_traffic(kernel, key + "_other") is None
    assert b._ncu_traffic("no_such_kernel", key) is None
