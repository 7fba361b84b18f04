"""bench.py's reference arm on the CPU: its one JSON line (metric, value,
unit, impl, cpu_baseline, e2e with zero transfer bytes) on a small grid, and
the silent exit of the non-zero ranks under a multi-rank launch."""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _bench(extra_env, *args):
    env = dict(os.environ)
    env.update(extra_env)
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_line():
    p = _bench({"WORLD_SIZE": "1", "RANK": "0"}, "--impl", "reference", "--n", "64", "--steps", "2", "--warmup", "1")
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "GB/s" and line["value"] > 0
    assert line["metric"].startswith("Jacobi HBM GB/s") and line["higher_is_better"] is True
    assert line["steps"] == 2 and line["warmup"] == 1 and line["n_gpus"] == 1
    assert "64^3" in line["config"]["workload"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    p = _bench({"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"}, "--impl", "reference", "--n", "64", "--steps",
               "1", "--warmup", "0", "--gpus", "2")
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
