"""bench.py's JSON line (CPU): the reference arm runs here on a small configuration and
prints one line with the keys the measurement contract names."""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "C1",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    b = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"):
        assert k in b, k
    assert b["impl"] == "reference" and b["dtype"] == "f64" and b["value"] > 0
    assert b["metric"] == b["unit"] == "DOF*RK-stage/s"
    assert b["cpu_baseline"]["value"] == b["value"] and b["cpu_baseline"]["cores"] >= 1
    assert b["cpu_baseline"]["kind"] in ("port", "reference")
    assert b["e2e"]["value"] == b["value"] and b["e2e"]["h2d_bytes_per_step"] == 0
    assert "workload" in b["config"] and "model" not in b["config"]
