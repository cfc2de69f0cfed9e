"""The CPU oracle against the reference's own known-answer tests
(lib/src/lib.rs:342-505 with the data of lib/src/test_data.rs:15-135) and the
single-colour tables of lib/src/colourfit/single_lut.rs (by SHA-256)."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

ALGOS = {"ClusterFit": 1, "RangeFit": 0, "IterativeClusterFit": 2}
FORMATS = {"BC1": 0, "BC2": 1, "BC3": 2, "BC4": 3, "BC5": 4}


def test_storage_requirements(oracle, kat):
    for c in kat["storage_requirements"]:
        assert oracle.compressed_size(FORMATS[c["format"]], c["width"], c["height"]) == c["size"]


@pytest.mark.parametrize("name", ["BC1_GRAY", "BC1_COLOUR", "BC2_GRAY", "BC2_COLOUR", "BC3_GRAY",
                                  "BC3_COLOUR", "BC4_GRAY", "BC5_GRAY"])
def test_compression_kat(oracle, kat, name):
    d = kat["datasets"][name]
    fmt = FORMATS[d["format"]]
    assert kat["compression_params"]["algorithms"] == ["ClusterFit", "RangeFit", "IterativeClusterFit"]
    for alg in kat["compression_params"]["algorithms"]:
        p = oracle.make_params(ALGOS[alg], kat["compression_params"]["weights"], False)
        out = oracle.compress(fmt, np.array(d["decoded"], np.uint8), 4, 4, p)
        assert out.tolist() == d["encoded"], (name, alg)


@pytest.mark.parametrize("name", ["BC1_GRAY", "BC1_COLOUR", "BC2_GRAY", "BC2_COLOUR", "BC3_GRAY",
                                  "BC3_COLOUR", "BC4_GRAY", "BC5_GRAY"])
def test_decompression_kat(oracle, kat, name):
    d = kat["datasets"][name]
    out = oracle.decompress(FORMATS[d["format"]], np.array(d["encoded"], np.uint8), 4, 4)
    assert out.tolist() == d["decoded"]


def test_bc1_decompression_height_not_multiple_of_4(oracle, kat):
    c = kat["odd_height_decode"]
    out = oracle.decompress(0, np.array(c["encoded"], np.uint8), c["width"], c["height"])
    assert out.reshape(-1, 4).tolist() == [c["pixel"]] * (c["width"] * c["height"])


def test_single_colour_tables_match_reference(oracle):
    with open(os.path.join(GOLDEN, "single_lut_sha256.json")) as f:
        digests = json.load(f)["sha256"]
    for i, name in enumerate(["LOOKUP_5_3", "LOOKUP_6_3", "LOOKUP_5_4", "LOOKUP_6_4"]):
        assert hashlib.sha256(oracle.single_lut(i).tobytes()).hexdigest() == digests[name], name


def test_lut_error_columns_regenerate(oracle):
    """Each error column is the distance to the nearest reachable 8-bit value
    (endpoints expanded as colourblock.rs:108-110, interpolants floored)."""
    for which, (bits, colours) in enumerate([(5, 3), (6, 3), (5, 4), (6, 4)]):
        t = oracle.single_lut(which).reshape(256, 2, 3)
        n = 1 << bits
        vals = [(v << (8 - bits)) | (v >> (2 * bits - 8)) for v in range(n)]
        reach = [set(), set()]
        for a in vals:
            for b in vals:
                reach[0].add(a)
                reach[1].add((a + b) // 2 if colours == 3 else (2 * a + b) // 3)
        for k in range(2):
            r = np.array(sorted(reach[k]))
            for target in range(256):
                assert t[target, k, 2] == np.abs(r - target).min()


def test_oracle_threading_is_deterministic(oracle):
    from texpresso_gb300 import workloads
    img = workloads.ramp_texture(96, 72, seed=5, alpha="ramp")
    for fmt in (0, 2):
        p = oracle.make_params(1, (0.2126, 0.7152, 0.0722), True)
        a = oracle.compress(fmt, img, 96, 72, p, nthreads=1)
        b = oracle.compress(fmt, img, 96, 72, p, nthreads=4)
        assert np.array_equal(a, b)
