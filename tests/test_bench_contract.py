"""The reference arm of bench.py on CPU: the JSON line it prints (one full-size step of the CPU
restatement), and the silent exit of ranks other than 0 under a multi-rank launch."""
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env):
    env = dict(os.environ, **extra_env)
    t0 = time.perf_counter()
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=900)
    out.wall_s = time.perf_counter() - t0
    return out


def test_reference_arm_line():
    out = _run({"RANK": "0", "WORLD_SIZE": "1"})
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "proofs/sec" and line["unit"] == "proofs/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["steps"] == 1 and line["warmup"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "proofs/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["num_vars"] == 22 and line["config"]["num_queries"] == 34
    # each step is a measured full-size proof: the timed steps fit inside the process's own run
    assert line["steps"] * line["ms_per_step"] / 1e3 <= out.wall_s
    assert len(line["step_ms_all"]) == line["steps"]


def test_reference_arm_other_ranks_exit_quietly():
    out = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""
