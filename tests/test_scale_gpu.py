"""Parity at the sizes the benchmark runs.

The bench's verify leg (bench.py verify_outputs) compares every output of one
timed step with the C oracle without copying the outputs back: triangle counts
and position-keyed checksums of every coords and normals word per 2^20
triangles (kvsmc_checksum_words on the device, mco_dup_checksum on the host).
  * 1024^3 float32 fBm, 16 isovalues (the headline sweep): the whole volume,
    634.8 M triangles, every triangle of every output.
  * 2048 x 2048 x 1024 uint16 stress volume, 4 isovalues (~1.1e9 triangles):
    the first and last two cell planes of every output, against the first and
    last triangles of each output (the last planes' node indices pass 2^32).
The reference's cell order is MarchingCubes.cpp:180-234.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(workload):
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--workload", workload, "--steps", "1", "--warmup", "3",
           "--no-cpu", "--no-e2e"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=1500)
    assert r.returncode == 0, r.stderr[-4000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    return line


def _check(line, n_iso):
    v = line["verify"]
    assert len(v["isolevels"]) == n_iso
    for e in v["isolevels"]:
        for sl in e["slabs"]:
            assert "first_diff" not in sl and "count_mismatch" not in sl, (e["isovalue"], sl)
    assert line["verified"] is True


def test_sweep1024_every_triangle_matches_the_oracle():
    line = _bench("sweep1024")
    _check(line, 16)
    assert sum(e["triangles"] for e in line["verify"]["isolevels"]) == line["triangles_per_step"]


def test_heavy_first_and_last_planes_match_the_oracle():
    line = _bench("heavy")
    _check(line, 4)
    for e in line["verify"]["isolevels"]:
        assert all(sl["triangles"] > 0 for sl in e["slabs"])
