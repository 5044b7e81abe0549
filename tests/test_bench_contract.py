"""bench.py's host-side contract, without a GPU: the reference arm (the CPU
oracle on the host cores) prints one JSON line with every key of the
benchmark line, and the algorithmic byte counts used by the roofline are the
documented per-element figures."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--nx", "12", "--steps", "2",
                          "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [x for x in out.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["metric"] == "cell-updates/s" and d["value"] > 0
    assert d["steps"] == 2 and d["warmup"] == 1 and d["higher_is_better"] is True
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert "workload" in d["config"]


def test_roofline_byte_counts():
    sys.path.insert(0, str(ROOT))
    import bench
    # FP64 kernel: 4 x 81 x 8 operators + 9 x 8 P/alpha + 18 x 8 x 2 + 4 x 2 x 8 velocity
    assert bench.bytes_per_element_iteration_stress(8) == 3016
    # FP32 operator-streaming kernels: 4 x 81 x 4 + 9 x 8 + 9 x 4 + 18 x 4 x 2 + 32
    assert bench.bytes_per_element_iteration_stress(4) == 1580
    # parallelogram kernel: 5 x 4 coefficients + 9 x 8 + 18 x 4 x 2 + 32 (P/(2 alpha) formed in-kernel)
    assert bench.bytes_per_element_iteration_stress(4, parallelogram=True) == 268
    # spherical FP32 kernel: 6 x 81 x 4 operators
    assert bench.bytes_per_element_iteration_stress(4, spherical=True) == 2228
