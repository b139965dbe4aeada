"""The reference arm of bench.py (``--impl reference``): the oracle's CPU
restatement of the reference's path, timed on the host cores, printing one
JSON line in the same form as the GPU arm -- same metric, unit and
direction, a ``cpu_baseline`` naming what ran, and an ``e2e`` with no host
copies.  Under torchrun only rank 0 runs; the other ranks exit 0 without
output.  Runs on the CPU (a small workload, one step)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None, *args):
    env = dict(os.environ)
    env.update(extra_env or {})
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "uniform2d",
                        "--steps", "1", "--warmup", "1", *args],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    return r


def test_reference_arm_line():
    pytest.importorskip("scipy")
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    import bench
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["steps"] == 1
    assert "2D type-1" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_reference_arm_batch_is_unavailable():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "batch64"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert d["impl"] == "reference" and "unavailable" in d
