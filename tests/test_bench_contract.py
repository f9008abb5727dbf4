"""bench.py's reference arm end to end on the CPU with a tiny sample: it prints one JSON
line with the keys of the bench contract (the GPU arm's line is checked on the GPU by the
same keys)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
        "cpu_baseline", "e2e"]


def test_reference_arm_prints_one_contract_line():
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--models", "2", "--packets",
           "2000", "--cpu-models", "2", "--cpu-packets", "2000", "--steps", "2", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["unit"] == "packets/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 0 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["seeds"]["mc_seeds"] == [0, 1] and len(d["seeds"]["ms_per_step"]) == 2
    assert d["interactions"]["per_s"] > 0
