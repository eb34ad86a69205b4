"""bench.py --impl reference on the host cores (no GPU): one JSON line with
the GPU arm's metric and unit, `impl: "reference"`, a cpu_baseline that
describes this run and an e2e equal to the value, as the driver reads it.
Run at 20,000 points (--n) so that the host builds the input table in
seconds; the arm's default is the full 1,024,000-point workload."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_prints_one_json_line():
    env = dict(os.environ, WORLD_SIZE="1", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0", "--n", "20000"], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    j = json.loads(lines[0])
    assert j["impl"] == "reference"
    assert j["metric"] == "fit_transform_seconds" and j["unit"] == "s"
    assert j["higher_is_better"] is False and j["steps"] == 1 and j["warmup"] == 0
    assert j["value"] > 0 and j["ms_per_step"] == j["value"] * 1000.0
    cb = j["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == j["value"]
    assert "points" in cb["sample"] and "no extrapolation" in cb["sample"]
    assert "not in the timed region" in j["config"]["knn"]
    assert j["e2e"] == {"value": j["value"], "unit": "s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert j["config"]["workload"].startswith("fit_transform N=20000 ")
