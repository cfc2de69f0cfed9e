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


def test_reference_arm_maps_no_product_library(built):
    """The reference arm times the CPU algorithm only: the GPU library must not
    even be mapped into its process."""
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--size', '64', '--steps', '3', "
            "'--warmup', '3']; import bench; bench.main(); maps = open('/proc/self/maps').read(); "
            "assert 'libtexpresso_gb300' not in maps, 'product library mapped'; "
            "assert 'libtexpresso_oracle' in maps; print('clean')")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().splitlines()[-1] == "clean"


def test_parity_record_counts_identical_ties_and_non_ties(oracle):
    """bench.py's oracle check of timed outputs: identical buffers count as
    identical, a flipped index bit in a bit-exact path (RangeFit) or in an
    alpha half is a non-tie."""
    sys.path.insert(0, ROOT)
    import bench
    from texpresso_gb300 import workloads
    img = workloads.ramp_texture(32, 16, seed=3, alpha="ramp")
    w = (0.2126, 0.7152, 0.0722)
    ref = oracle.compress(2, img, 32, 16, oracle.make_params(1, w, False))
    rec = bench.oracle_parity(oracle, 2, img, 1, w, False, [ref.copy(), ref.copy()])
    assert rec["blocks"] == 64 and rec["identical"] == 64 and rec["identical_fraction"] == 1.0
    assert rec["ties"] == 0 and rec["non_ties"] == 0
    bad = ref.copy().reshape(-1, 16)
    bad[5, 3] ^= 0x01  # alpha index bits of block 5
    rec = bench.oracle_parity(oracle, 2, img, 1, w, False, [bad.reshape(-1)])
    assert rec["identical"] == 31 and rec["non_ties"] == 1
    rref = oracle.compress(2, img, 32, 16, oracle.make_params(0, w, False))
    bad = rref.copy().reshape(-1, 16)
    bad[7, 12] ^= 0x04  # a colour index of a RangeFit block
    rec = bench.oracle_parity(oracle, 2, img, 0, w, False, [bad.reshape(-1)])
    assert rec["non_ties"] == 1 and rec["ties"] == 0
