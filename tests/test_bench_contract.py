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
    # the same config dict as the GPU arm's (bench.config_dict), window included
    assert b["config"]["window"] == "steps 1000-1000 of the 1000-step run"
    for k in ("cells", "N", "dof", "stages_per_step", "l2", "parallelism"):
        assert k in b["config"], k


def test_clock_summary_reads_nvidia_smi_samples():
    """The `clocks` object of the GPU line: median SM clock under load, the maximum, and
    every throttle reason seen Active in any sample (the ones that reject a run among
    them); malformed or partial lines are skipped."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    clk = bench.ClockSampler(0)
    clk.lines = [
        "0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 1950, 2070, 1390.5, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1000.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, [N/A], 2070, 10.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2070, 2070",
    ]
    s = clk.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    clk.lines = ["0, 1200, 2070, 700, 0x8, Not Active, Active, Not Active, Not Active"]
    assert clk.summary()["reasons"] == ["hw_thermal_slowdown"]
    clk.lines = []
    assert clk.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
