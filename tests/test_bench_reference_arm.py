"""bench.py --impl reference (no GPU): the reference's CPU algorithm (the
oracle port) over steps W ... W+K-1 of its own FP64 trajectory prints one
JSON line with the contract's keys, an e2e object with no copies and a
cpu_baseline describing the run."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3", "--ref-max-steps", "1"],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    r = json.loads(lines[0])
    assert r["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in r, k
    assert r["value"] > 0 and r["higher_is_better"] is True and r["warmup"] >= 3
    assert r["config"]["workload"] == "disk16k"
    cb = r["cpu_baseline"]
    assert cb["value"] == r["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    assert "sample" in cb
    e2e = r["e2e"]
    assert e2e["value"] == r["value"] and e2e["unit"] == r["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
