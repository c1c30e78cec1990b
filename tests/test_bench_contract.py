"""bench.py's output contract: the reference arm (the CPU restatement of the
path) prints one JSON line with the keys the measurement harness reads -- on
the CPU for the single-pair workload, on the GPU machine for the default
workload, whose inputs a child process renders -- and the argument parser
knows every workload."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _reference_line(*extra):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
                        *extra], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["unit"] == "pairs/s" and d["steps"] == 1
    assert d["value"] >= 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"]
    return d


def test_reference_arm_prints_one_json_line():
    _reference_line("--workload", "config1")


@pytest.mark.gpu
def test_reference_arm_of_the_default_workload():
    d = _reference_line()
    assert d["config"]["workload"].startswith("config 4") and d["config"]["pairs_timed"] == 1


def test_workloads_are_listed_in_the_help():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True, text=True, timeout=120,
                       cwd=ROOT)
    assert r.returncode == 0
    for w in ("config4", "config1", "turntable36", "proposal", "sfm", "sr"):
        assert w in r.stdout, w
