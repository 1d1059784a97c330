"""The benchmark's JSON-line assembly on CPU: every secondary workload line
carries the contract keys, and a line without a CPU baseline (the H64
k-point workload records why it has none) is assembled as well as one with
it."""
import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_line_with_and_without_cpu_baseline():
    sys.path.insert(0, ROOT)
    import bench
    args = argparse.Namespace(steps=8, warmup=3)
    keys = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
            "scaling", "vs_baseline", "data", "config"}
    none = bench._line("m", "evals/s", 1.0, 2.0, args, {"workload": "w"},
                       {"cpu_baseline": None, "cpu_baseline_note": "not run"})
    assert keys <= set(none) and none["cpu_baseline"] is None
    some = bench._line("m", "evals/s", 1.0, 2.0, args, {"workload": "w"},
                       {"cpu_baseline": {"value": 0.5, "unit": "evals/s", "kind": "port"}})
    assert some["cpu_baseline"]["cores"] >= 1
    json.dumps(none), json.dumps(some)
