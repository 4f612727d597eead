"""bench.py --impl reference (the reference's CPU algorithm, restated in
oracle/, on the host cores) keeps the bench line's contract: one JSON line
from rank 0 with the arm's metric, unit, cpu_baseline and a copy-free e2e;
other ranks print nothing and exit 0.  A small disk is timed whole."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CMD = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "disk64",
       "--steps", "2", "--warmup", "3"]


def test_reference_arm_line():
    out = subprocess.run(CMD, capture_output=True, text=True, timeout=600, cwd=ROOT, check=True)
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for key in ("metric", "unit", "value", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "dtype", "data", "config"):
        assert key in d, key
    assert d["steps"] == 2 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["value"] > 0 and abs(d["ms_per_step"] - 1e3 / d["value"]) <= 1e-6 * d["ms_per_step"]
    assert d["config"]["workload"].startswith("disk64")
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "disk64" in cb["sample"]
    assert cb["host"]["nproc"] >= cb["cores"] and cb["host"]["model"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_are_silent():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run(CMD, capture_output=True, text=True, timeout=600, cwd=ROOT, env=env)
    assert out.returncode == 0
    assert not [l for l in out.stdout.splitlines() if l.startswith("{")]
