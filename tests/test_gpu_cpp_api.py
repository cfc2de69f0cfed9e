"""The C++ mirror of the reference API (include/texpresso.hpp) runs the
reference's own unit tests (lib/src/lib.rs:342-505) on the GPU."""
import json
import os
import subprocess

import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu


def _kat_header(path):
    kat = json.load(open(os.path.join(GOLDEN, "kat.json")))
    fmt = {"BC1": 0, "BC2": 1, "BC3": 2, "BC4": 3, "BC5": 4}
    out = ["#pragma once", "#include <cstdint>", "#include <cstddef>",
           "struct KatSet { int format; const uint8_t *encoded; size_t encoded_len; const uint8_t *decoded; };"]
    names = []
    for name, d in kat["datasets"].items():
        out.append("static const uint8_t %s_ENC[] = {%s};" % (name, ",".join(map(str, d["encoded"]))))
        out.append("static const uint8_t %s_DEC[] = {%s};" % (name, ",".join(map(str, d["decoded"]))))
        names.append("{%d, %s_ENC, sizeof(%s_ENC), %s_DEC}" % (fmt[d["format"]], name, name, name))
    out.append("static const KatSet KAT_SETS[] = {%s};" % ", ".join(names))
    odd = kat["odd_height_decode"]
    out.append("static const uint8_t ODD_ENCODED[] = {%s};" % ",".join(map(str, odd["encoded"])))
    out.append("static const uint8_t ODD_PIXEL[] = {%s};" % ",".join(map(str, odd["pixel"])))
    open(path, "w").write("\n".join(out) + "\n")


def test_reference_unit_tests_in_cpp(tx, cuda, tmp_path):
    _kat_header(str(tmp_path / "kat_data.h"))
    exe = str(tmp_path / "test_reference_api")
    libdir = os.path.dirname(tx.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", str(tmp_path),
                    os.path.join(ROOT, "tests", "cpp", "test_reference_api.cpp"), "-L", libdir,
                    "-ltexpresso_gb300", "-Wl,-rpath," + libdir, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
