"""The reference arm of bench.py on the CPU: one JSON line with the keys the
benchmark contract names (metric, value, unit, steps, warmup, impl, config,
cpu_baseline, e2e with no host transfers), on a small heat step."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_reference(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *args],
                         cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def test_reference_arm_prints_the_contract_line():
    d = run_reference("--elements", "16", "--steps", "3", "--warmup", "3")
    assert d["impl"] == "reference"
    assert d["unit"] == "DOF-updates/s" and d["higher_is_better"] is True
    assert d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["config"]["elements"] == [16, 16, 16] and d["config"]["degree"] == 2
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # the DOFs of one step of the sample: (16 + 2)^3 at p = 2
    assert d["config"]["dofs_per_step"] == 18 ** 3
