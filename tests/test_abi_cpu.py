"""The C-ABI library without a GPU: it loads, exports every entry point the
public headers declare, and rejects the arguments the reference panics on
(lib/src/lib.rs:295, slice bounds) before touching a device."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_symbols():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        names += re.findall(r"TX_API\s+[\w\s\*]+?\b(tx_\w+)\s*\(", src)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("tx_compress", "tx_compress_block_masked", "tx_compress_device", "tx_decompress",
              "tx_decompress_block", "tx_compressed_size", "tx_block_size", "tx_params_default"):
        assert n in names


def test_library_exports_every_declared_symbol(tx):
    lib = ctypes.CDLL(tx.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_only_tx_symbols_exported(tx):
    out = os.popen("nm -D --defined-only %s" % tx.LIB_PATH).read().split("\n")
    syms = [l.split()[-1] for l in out if l.strip() and l.split()[1] in ("T", "D", "B")]
    own = [s for s in syms if not s.startswith("tx_")]
    # the static CUDA runtime may export nothing of its own; our code exports tx_* only
    assert all(not s.startswith("_ZN2tx") for s in own), own


def test_params_default_matches_reference(tx):
    p = tx._CParams()
    tx.library().tx_params_default(ctypes.byref(p))
    assert p.algorithm == 1  # Algorithm::ClusterFit (lib.rs:61-65)
    assert list(p.weights) == list(np.array([0.2126, 0.7152, 0.0722], np.float32))
    assert p.weigh_colour_by_alpha == 0
    d = tx.Params()
    assert d.algorithm == tx.Algorithm.ClusterFit and tuple(d.weights) == tx.COLOUR_WEIGHTS_PERCEPTUAL


def test_sizes_match_reference(tx, kat):
    for c in kat["storage_requirements"]:
        f = tx.Format[c["format"].capitalize()]
        assert f.compressed_size(c["width"], c["height"]) == c["size"]
    assert [tx.Format(i).block_size() for i in range(5)] == [8, 16, 16, 8, 16]
    assert tx.library().tx_block_size(7) == 0
    assert [tx.num_blocks(s) for s in (0, 1, 4, 5, 8)] == [0, 1, 1, 2, 2]


def rc_compress(tx, fmt, rgba_len, w, h, out_len, algorithm=1):
    rgba = np.zeros(max(rgba_len, 1), np.uint8)
    out = np.zeros(max(out_len, 1), np.uint8)
    p = tx._CParams()
    tx.library().tx_params_default(ctypes.byref(p))
    p.algorithm = algorithm
    return tx.library().tx_compress(fmt, rgba.ctypes.data, rgba_len, w, h, ctypes.byref(p), out.ctypes.data, out_len)


def test_argument_errors_without_device(tx):
    lib = tx.library()
    assert rc_compress(tx, 9, 64, 4, 4, 8) == -1                  # invalid format
    assert rc_compress(tx, 0, 64, 0, 4, 8) == -2                  # width 0: chunk size 0 panics
    assert rc_compress(tx, 0, 64, 4, 4, 4) == -3                  # lib.rs:295 assert
    assert rc_compress(tx, 0, 64, 4, 4, 12) == -2                 # trailing partial block panics
    assert rc_compress(tx, 0, 60, 4, 4, 8) == -4                  # input slice too short
    assert rc_compress(tx, 0, 64, 4, 4, 8, algorithm=7) == -2     # no such algorithm
    assert rc_compress(tx, 2, 64, 4, 4, 8) == -3                  # BC3 needs 16 bytes
    assert rc_compress(tx, 0, 0, 4, 0, 0) == 0                    # empty image: nothing to do
    for s in (-1, -2, -3, -4, -5, -6, -7):
        assert lib.tx_status_string(s).decode() != "unknown status"


def test_python_mirror_raises_where_reference_panics(tx):
    with pytest.raises(tx.TexpressoError) as e:
        tx.Format.Bc1.compress(bytes(64), 4, 4, tx.Params(), bytearray(4))
    assert e.value.status == -3
    with pytest.raises(tx.TexpressoError) as e:
        tx.Format.Bc1.compress(bytes(64), 0, 4, tx.Params(), bytearray(8))
    assert e.value.status == -2


def test_no_cpu_fallback_without_device(tx):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(tx.TexpressoError) as e:
        tx.Format.Bc1.compress(bytes(64), 4, 4, tx.Params(), bytearray(8))
    assert e.value.status == -6


def test_batch_rejects_bad_items_without_device(tx):
    buf = np.zeros(1024, np.uint8)
    ok = tx.batch_item(0, buf.ctypes.data, 16, 4, 4, tx.Params(), buf.ctypes.data)
    bad_fmt = tx.batch_item(9, buf.ctypes.data, 16, 4, 4, tx.Params(), buf.ctypes.data)
    bad_ch = tx.batch_item(0, buf.ctypes.data, 16, 4, 4, tx.Params(), buf.ctypes.data, channels=2)
    bad_pitch = tx.batch_item(0, buf.ctypes.data, 8, 4, 4, tx.Params(), buf.ctypes.data)
    bad_align = tx.batch_item(2, buf.ctypes.data, 16, 4, 4, tx.Params(), buf.ctypes.data + 8)
    for item, status in ((bad_fmt, -1), (bad_ch, -2), (bad_pitch, -2), (bad_align, -9)):
        with pytest.raises(tx.TexpressoError) as e:
            tx.Batch([ok, item])
        assert e.value.status == status
    assert tx.mip_count(0, 5) == 0 and tx.mip_count(1, 1) == 1 and tx.mip_count(4096, 2) == 13


def test_mip_reference_definition():
    from texpresso_gb300 import workloads
    img = np.arange(5 * 3 * 4, dtype=np.uint8).reshape(3, 5, 4)
    m = workloads.mip_reference(img)
    assert m.shape == (1, 2, 4)
    a = img.astype(int)
    assert m[0, 1, 0] == (a[0, 2, 0] + a[0, 3, 0] + a[1, 2, 0] + a[1, 3, 0] + 2) >> 2


def test_server_needs_a_device(tx):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(tx.TexpressoError) as e:
        tx.Server(memory_budget=1 << 20)
    assert e.value.status == -6
    assert tx.chain_compressed_size(0, 4, 4, False) == 8
    assert tx.chain_compressed_size(0, 8, 8, True) == 8 * 4 + 8 + 8 + 8  # 8x8, 4x4, 2x2, 1x1
    assert tx.chain_compressed_size(9, 8, 8, True) == 0
