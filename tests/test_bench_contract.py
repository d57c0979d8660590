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


def test_double_float_operation_model():
    """The roofline's operation count of the double-float assembly: the
    direct sums at p = 2 (8,187 FP32 operations per element), fewer with the
    even-odd form, and the fractions of the work in that form at 256^3 (every
    x brick but the two holding an end element, every row and layer but the
    two end ones) and at 96^3 (FP32-rounded knots: no whole brick)."""
    sys.path.insert(0, ROOT)
    import bench
    from ads_mpi_gb300 import ads as A
    assert bench.df_assembly_ops(2, 1) == 8187
    assert bench.df_assembly_ops(2, 1, (1.0, 1.0, 1.0)) < 0.81 * 8187
    assert bench.df_assembly_ops(2, 1, (1.0, 1.0, 1.0), fold=True) < bench.df_assembly_ops(2, 1, (1.0, 1.0, 1.0))
    # constant conductivity: the x stage is three banded products per row of
    # points and DOF column, whatever the symmetry (166 operations at p = 2)
    assert bench.df_assembly_ops(2, 1, fold=True) - bench.df_assembly_ops(2, 1, (1.0, 0.0, 0.0), fold=True) == 0
    assert bench.df_assembly_ops(2, 1, (1.0, 1.0, 1.0), fold=True) < 0.41 * 8187
    fx, fy, fz = bench.even_odd_fractions(A, 256, 2)
    assert fx == (256 - 30 - 16) / 256 and fy == fz == 254 / 256
    fx96, fy96, _ = bench.even_odd_fractions(A, 96, 2)
    assert fx96 == 0.0 and 0.0 < fy96 < 1.0
    assert bench.even_odd_fractions(A, 256, 3) == (0.0, 0.0, 0.0)
