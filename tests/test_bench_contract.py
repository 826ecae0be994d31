"""CPU checks of bench.py's output contract.

The reference arm (the reference algorithm on the host cores) runs without a
GPU, so its JSON line can be checked here at a small size: one line on
stdout with the keys, types and units every bench line carries.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

BASE_KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
             "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"}


def run_reference_arm(*extra):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--ref-n", "384", "--steps", "2", "--warmup", "1", *extra],
                         cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def test_reference_arm_line():
    d = run_reference_arm()
    assert BASE_KEYS <= set(d), BASE_KEYS - set(d)
    assert d["impl"] == "reference"
    assert d["metric"].startswith("dgeqp4 TFLOP/s")
    assert d["unit"] == "TFLOP/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    # value = (2 m n^2 - 2 n^3 / 3) / time for the m = n = 384 sample.
    n = 384
    flops = 2.0 * n * n * n - 2.0 * n ** 3 / 3.0
    assert abs(d["value"] - flops / (d["ms_per_step"] * 1e-3) / 1e12) <= 1e-6 * d["value"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1
    assert isinstance(cb["cpu_model"], str) and cb["cpu_model"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert d["config"]["m"] == d["config"]["n"] == n
