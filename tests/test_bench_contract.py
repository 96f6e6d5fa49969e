"""The bench's CPU-side lines: the reference arm (`--impl reference`, the
oracle on the host cores) and the CPU-baseline child (`--cpu-baseline-only`)
print one JSON line with the keys the measurement contract names, without a
GPU."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _last_json(args):
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py")] + args, capture_output=True,
                         text=True, check=True, timeout=300, cwd=REPO).stdout
    return json.loads(out.strip().splitlines()[-1])


def test_reference_arm_line(oracle_mod):
    d = _last_json(["--impl", "reference", "--workload", "uniform_64k", "--steps", "2", "--warmup", "1"])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == "body-steps/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 1 and d["value"] > 0
    assert d["config"]["workload"] == "uniform_64k"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_cpu_baseline_child_line(oracle_mod):
    d = _last_json(["--cpu-baseline-only", "--workload", "uniform_64k", "--cpu-seconds", "0.3"])
    assert d["unit"] == "body-steps/s" and d["value"] > 0
    assert d["kind"] == "port" and d["cores"] >= 1 and "sample" in d
    assert d["single_thread"]["value"] > 0
