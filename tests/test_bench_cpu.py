"""Host-side pieces of bench.py that need no GPU: the DRAM-traffic table the
roofline's `traffic` comes from, and its lookup by workload, size and kernel."""
import importlib.util
import json
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_traffic_table_entries_are_complete():
    with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as fh:
        d = json.load(fh)
    entries = {k: v for k, v in d.items() if not k.startswith("_")}
    assert entries
    for key, e in entries.items():
        assert e["dram_bytes_per_update"] > 0, key
        assert e["capture"].startswith("ncu ") and "--clock-control none" in e["capture"], key
        assert "bench.py" in e["capture"], key
        assert e["kernel"] and e["captured"], key


def test_traffic_lookup_by_kernel():
    b = _bench()
    with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as fh:
        d = json.load(fh)
    # the cluster kernel's entry carries no kernel suffix, the tiled one does
    t, cap = b._traffic("batch512_pt:L48", 1000.0)
    assert t == d["batch512_pt:L48"]["dram_bytes_per_update"] * 1000.0 and cap
    t, cap = b._traffic("batch512_pt:L48:tile", 1000.0)
    assert t == d["batch512_pt:L48:tile"]["dram_bytes_per_update"] * 1000.0 and cap
    assert b._traffic("no such workload", 1.0) == (None, None)
