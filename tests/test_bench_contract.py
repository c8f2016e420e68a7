"""bench.py's reference arm against the benchmark line contract (CPU: the arm times the oracle).

The arm runs rank 0 only; its line carries the arm's own metric/config, a cpu_baseline that
describes the run and an e2e object with no host<->device traffic."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

REQUIRED = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e")


def _bench(env=None):
    return subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                          cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)


def test_reference_arm_json_line():
    out = _bench()
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for k in REQUIRED:
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["steps"] == 1 and line["warmup"] == 0 and line["n_gpus"] == 1
    assert line["higher_is_better"] is True and line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["workload"].startswith("large blend 128^3")
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["value"] == line["value"] and cb["cores"] >= 1
    assert cb["unit"] == line["unit"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    out = _bench(env=dict(os.environ, RANK="1", WORLD_SIZE="2"))
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""
