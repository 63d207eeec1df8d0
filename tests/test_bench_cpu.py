"""bench.py's reference arm runs on host cores alone: its JSON line carries the
fields the benchmark contract names (impl, metric and unit of the workload,
a cpu_baseline describing the run, an e2e entry with no host-device bytes)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_line(workload):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--workload", workload],
                         cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line():
    d = _reference_line("blobs128")
    assert d["impl"] == "reference"
    assert d["metric"] == "Mcells/s" and d["unit"] == "Mcells/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] >= 3
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert cb["cores"] == 1   # one isovalue: one thread works
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in d["config"] and "sample" in d["config"]


def test_reference_arm_times_the_workloads_mode():
    d = _reference_line("blobs128vn")
    assert "VertexNormal" in d["config"]["sample"] and d["value"] > 0


@pytest.mark.parametrize("workload,metric", [("kvsml512", "GB/s"), ("stlascii512", "Mtris/s")])
def test_reference_arm_uses_the_workloads_metric(workload, metric):
    d = _reference_line(workload)
    assert d["metric"] == metric and d["unit"] == metric and d["value"] > 0
    assert d["cpu_baseline"]["unit"] == metric and d["e2e"]["unit"] == metric
