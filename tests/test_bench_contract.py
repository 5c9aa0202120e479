"""bench.py's reference arm runs on the host cores (no GPU) and prints the one JSON
line the benchmark contract asks for."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    x = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"):
        assert key in x, key
    assert x["impl"] == "reference"
    assert x["steps"] == 1 and x["warmup"] == 3 and x["value"] > 0
    assert x["metric"] == "kron-matvec GFLOP/s" and x["higher_is_better"] is True
    assert x["e2e"]["value"] == x["value"] and x["e2e"]["h2d_bytes_per_step"] == 0
    assert x["cpu_baseline"]["kind"] in ("port", "reference") and x["cpu_baseline"]["cores"] >= 1
