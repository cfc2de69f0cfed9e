"""Exact integer pieces of texpresso_gb300/csrc/tx_device.cuh compiled for
the host with nvcc and checked exhaustively on the CPU: the alpha codebook
builders (make_book5 / make_book7) over the books' range pairs, against the
books' sorted-merge definition and the reference's first-minimum code search
(lib/src/alpha.rs:79-117); and the block coordinates by a precomputed
reciprocal (set_blocks_wide / block_coords) against plain division."""
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


def test_block_coords_on_the_host(tmp_path):
    """set_blocks_wide / block_coords (tx_device.cuh) against plain division."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "test_block_coords")
    subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "texpresso_gb300", "csrc"),
                    "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "test_block_coords.cu"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
