"""bench.py --impl reference on the CPU: the reference arm (the oracle's
restatement of the reference on every host thread) prints the one JSON line
the bench contract asks for, on a small sample of the point-flux workload."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "c1", "--steps", "1", "--warmup", "0", "--ref-rows", "8",
                        "--ref-events", "2000"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "cells/s" and d["value"] > 0
    for k in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config"):
        assert k in d, k
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "cells/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    ph = d["cpu_phases"]
    assert ph["events_sample"] == 2000 and ph["events_per_s_1_thread"] > 0
    assert ph["lumi_cells_per_s"] > 0 and ph["init_s"] > 0 and ph["fold_and_samplers_s"] > 0
    assert "c1: Pb-Pb 201x61" in d["config"]["workload"]
