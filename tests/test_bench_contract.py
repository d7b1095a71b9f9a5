"""bench.py's reference arm on the host: the one JSON line it prints (the
reference algorithm timed on the CPU cores, with the keys the benchmark's
readers expect), and its silence on ranks other than 0 under torchrun.
The GPU arm is covered by the GPU tests and the bench runs themselves."""

import json
import os
import subprocess
import sys

from conftest import ROOT


def run_bench(args, env_extra=None):
    env = dict(os.environ, **(env_extra or {}))
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_one_contract_line():
    out = run_bench(["--impl", "reference", "--steps", "2", "--warmup", "1", "--cpu-sample-rays", "512"])
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference"
    assert j["metric"] == "rays/s" and j["unit"] == "rays/s" and j["higher_is_better"] is True
    assert j["n_gpus"] == 1 and j["steps"] == 2 and j["warmup"] == 1
    assert j["value"] > 0 and j["ms_per_step"] > 0
    assert "workload" in j["config"] and "256x256" in j["config"]["workload"]
    cb = j["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == j["value"] and cb["unit"] == j["unit"]
    # a strided subset of the image: about the requested rays per step
    assert "rays per step" in cb["sample"] and 512 <= int(cb["sample"].split()[0]) < 1024
    e2e = j["e2e"]
    assert e2e["value"] == j["value"] and e2e["unit"] == j["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_without_work():
    out = run_bench(["--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1"],
                    {"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert out.returncode == 0, out.stderr[-2000:]
    assert not [l for l in out.stdout.splitlines() if l.startswith("{")]
