"""The reference arm of bench.py on CPU: `--impl reference` times the oracle
(the CPU restatement of the reference's DG tendency + LSRK54) on the full
rising-bubble workload and prints one JSON line with the arm's contract
keys; under a multi-rank launch only rank 0 prints."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_bench(env_extra, *args):
    env = dict(os.environ, **env_extra)
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", *args],
                         cwd=REPO, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return [l for l in out.stdout.splitlines() if l.strip()]


def test_reference_arm_line():
    lines = run_bench({}, "--steps", "2", "--warmup", "1")
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == "DOF-stage updates/s" and line["unit"] == "DOF-stage/s"
    assert line["higher_is_better"] is True
    assert line["steps"] == 2 and line["warmup"] == 1
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "DOF-stage/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    # the same config keys as the GPU arm, so the two lines describe one workload
    assert set(line["config"]) == {"workload", "l2", "parallelism"}


def test_reference_arm_other_ranks_exit_quietly():
    assert run_bench({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--steps", "1", "--warmup", "1") == []
