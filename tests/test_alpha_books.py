"""The alpha codebook builders (make_book5 / make_book7 in
texpresso_gb300/csrc/tx_device.cuh) compiled for the host with nvcc and
checked exhaustively over the books' range pairs: against the books'
sorted-merge definition and the reference's first-minimum code search
(lib/src/alpha.rs:79-117).  Runs on the CPU."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_alpha_books_on_the_host(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "test_alpha_books")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "texpresso_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_alpha_books.cu"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
