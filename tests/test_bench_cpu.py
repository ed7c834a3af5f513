"""bench.py's reference arm runs on the host cores alone: it times whole
fit_predict steps of the CPU port, never loads the engine's library, keeps
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


# Runs bench.py's reference arm in this interpreter, then reports whether the
# engine's library was ever mapped into the process.
PROBE = """
import runpy, sys
sys.argv = ["bench.py"] + sys.argv[1:]
try:
    runpy.run_path(sys.argv[0], run_name="__main__")
except SystemExit as e:
    assert not e.code, e.code
maps = open("/proc/self/maps").read()
print("ENGINE_LOADED" if "libculof_gb300" in maps else "ENGINE_NOT_LOADED")
"""


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, "-c", PROBE, "--impl", "reference", "--n", "3000", "--steps", "2",
                          "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    assert lines[-1] == "ENGINE_NOT_LOADED"
    line = json.loads(lines[-2])
    assert line["impl"] == "reference"
    assert line["metric"] == "pair-dists/s" and line["unit"] == "pair-dists/s"
    assert line["higher_is_better"] is True and line["scaling"] == "weak"
    assert line["steps"] == 2 and line["warmup"] == 1 and line["n_gpus"] == 1
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert line["config"]["n"] == 3000 and "workload" in line["config"]
    assert "path" not in line["config"]  # the GPU arm's config dict has the same keys
    # whole steps, measured: the timed steps' mean is the line's time
    assert abs(line["ms_per_step"] - line["fit_predict_s"] * 1e3) < 1e-6
    assert abs(line["value"] - 3000.0 ** 2 / line["fit_predict_s"]) < 1e-6 * line["value"]
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
