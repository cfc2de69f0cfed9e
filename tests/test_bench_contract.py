"""The benchmark's reference arm (the reference's CPU algorithm on the host
cores) runs without a GPU: its JSON line carries every key of the bench
contract, and ranks other than 0 exit quietly.  Also checks that the work
unit the FP32 roofline counts matches the candidate lists the kernels use."""
import json
import os
import subprocess
import sys

from conftest import ROOT

KEYS = ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"]


def run_bench(args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + args, capture_output=True, text=True,
                          env=e, cwd=ROOT, timeout=600)


def test_reference_arm_line(built):
    r = run_bench(["--impl", "reference", "--size", "64", "--steps", "3", "--warmup", "3"])
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in KEYS:
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 3 and line["warmup"] == 3
    assert line["config"]["width"] == 64 and "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_exit_quietly(built):
    r = run_bench(["--impl", "reference", "--size", "64", "--steps", "3", "--warmup", "3"], env={"RANK": "1"})
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_roofline_work_unit_matches_candidate_lists():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.n4(16) == 967 and bench.n3(16) == 151
    assert bench.n4(8) == 163 and bench.n3(8) == 43
