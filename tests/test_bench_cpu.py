"""bench.py's reference arm runs on the host cores alone: its JSON line keeps
the benchmark contract (the same metric, unit and config keys as the GPU
arm), and under torchrun only rank 0 measures and prints."""

from __future__ import annotations

import json
import os
import subprocess
import sys

from conftest import ROOT

BENCH = os.path.join(ROOT, "bench.py")


def run_bench(args, extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    return subprocess.run([sys.executable, BENCH, *args], capture_output=True, text=True, timeout=300, env=env)


def test_reference_arm_json_line():
    out = run_bench(["--impl", "reference", "--n", "3000", "--steps", "2", "--warmup", "1", "--cpu-seconds", "0.2"])
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "pair-dists/s" and line["unit"] == "pair-dists/s"
    assert line["higher_is_better"] is True and line["scaling"] == "weak"
    assert line["steps"] == 2 and line["warmup"] == 1 and line["n_gpus"] == 1
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["n"] == 3000 and "workload" in line["config"]
    cpu = line["cpu_baseline"]
    assert cpu["value"] == line["value"] and cpu["cores"] >= 1 and cpu["kind"] in ("reference", "port") and cpu["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly():
    out = run_bench(["--impl", "reference", "--n", "3000", "--steps", "1", "--warmup", "1"],
                    {"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"})
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""
