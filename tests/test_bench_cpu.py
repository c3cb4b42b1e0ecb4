"""bench.py on the CPU: the timed kernel family per workload, and the
reference arm's JSON line (the C restatement of the reference step on the
host cores; it needs no GPU)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _parse(argv):
    sys.path.insert(0, ROOT)
    import bench
    old = sys.argv
    try:
        sys.argv = ["bench.py"] + argv
        return bench.parse()
    finally:
        sys.argv = old


def test_kernel_family_default_per_workload():
    assert _parse([]).kernel == "fast"
    assert _parse(["--workload", "porous4m"]).kernel == "fast"
    assert _parse(["--workload", "cavity"]).kernel == "auto"
    assert _parse(["--workload", "channel"]).kernel == "auto"
    assert _parse(["--workload", "porous1m", "--kernel", "fused_nodes"]).kernel == "fused_nodes"
    assert _parse([]).check_time is None  # each workload picks its residual window


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "cavity", "--steps", "2", "--warmup", "1"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "MCUPS" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "MCUPS", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["higher_is_better"] is True and line["config"]["cells"] > 1000
