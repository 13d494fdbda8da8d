"""bench.py's line contract on the host: the compact summary of a workload's line, and the
default run's other workloads, where a failing workload is reported in its own slot and
the others still run (so the headline line always prints)."""
import argparse
import sys

from conftest import ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _line(value):
    return {"metric": "m", "value": value, "unit": "queries/s", "steps": 5, "warmup": 3, "ms_per_step": 1.0,
            "parity_checked": 2, "gpu_launches": 10, "config": {"workload": "w", "shards": 4},
            "e2e": {"value": value / 2, "unit": "queries/s", "h2d_bytes_per_step": 1},
            "clocks": {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 5, "region_s": 0.3},
            "saturation": {"queries_per_s": value}, "unrelated": [1, 2, 3]}


def test_compact_keeps_the_reported_fields():
    out = bench.compact(_line(100.0), 1.234)
    assert out["value"] == 100.0 and out["e2e"] == {"value": 50.0, "unit": "queries/s"}
    assert out["config"] == "w" and out["parity_checked"] == 2 and out["gpu_launches"] == 10
    assert out["clocks"] == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 5}
    assert out["saturation"] == {"queries_per_s": 100.0} and "unrelated" not in out
    assert out["wall_s"] == 1.2


def test_a_failing_workload_is_reported_in_its_slot(monkeypatch):
    seen = []

    def ok(args, rank, world):
        seen.append((args.workload, args.steps, args.lanes))
        return _line(float(len(seen)))

    def fails(args, rank, world):
        seen.append((args.workload, args.steps, args.lanes))
        raise RuntimeError("served response differs from the oracle")

    for name in ("run_sm", "run_cfg5", "run_tree", "run_nopack"):
        monkeypatch.setattr(bench, name, ok)
    monkeypatch.setattr(bench, "run_cfg4", fails)
    args = argparse.Namespace(workload="served-batch", steps=20, warmup=3, lanes=4, shards=bench.NUM_SHARDS,
                              requests=16384, no_cpu_baseline=True)
    out = bench.other_workloads(args, 0, 1)
    assert list(out) == list(bench.OTHER_WORKLOADS)
    assert "oracle" in out["mixed"]["error"] and "value" not in out["mixed"]
    assert all("value" in out[k] for k in out if k != "mixed")
    # Each workload runs at its own default steps and lanes.
    assert seen == [(w, bench.DEFAULT_STEPS[w], bench.DEFAULT_LANES.get(w, 3)) for w in bench.OTHER_WORKLOADS]
