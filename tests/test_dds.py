"""DDS container (tx_dds_*): the header the reference CLI writes through
ddsfile's new_dxgi (cli/src/main.rs:143-164) and the formats its
decompress_file accepts (cli/src/main.rs:167-248).  Host only."""
import struct

import numpy as np
import pytest

DXGI = {0: 72, 1: 75, 2: 78, 3: 80, 4: 83}


def test_header_layout(tx):
    for fmt in range(5):
        h = tx.dds_header(fmt, 15, 9)
        assert len(h) == 148 and h[:4] == b"DDS "
        size, flags, height, width, linear, depth, mips = struct.unpack_from("<7I", h, 4)
        assert size == 124 and (height, width) == (9, 15) and depth == 0 and mips == 0
        assert flags == 0x1 | 0x2 | 0x4 | 0x1000 | 0x80000          # caps, height, width, pixelformat, linearsize
        assert linear == tx.Format(fmt).compressed_size(15, 9)
        assert h[4 + 28:4 + 72] == bytes(44)                          # reserved1
        pf_size, pf_flags, fourcc = struct.unpack_from("<3I", h, 4 + 72)
        assert (pf_size, pf_flags, fourcc) == (32, 0x4, struct.unpack("<I", b"DX10")[0])
        caps, caps2 = struct.unpack_from("<2I", h, 4 + 104)
        assert caps == 0x1000 and caps2 == 0
        dxgi, dim, misc, array, alpha = struct.unpack_from("<5I", h, 128)
        assert dxgi == DXGI[fmt] and dim == 3 and misc == 0 and array == 1
        assert alpha == (2 if fmt == 0 else 1)                        # premultiplied for BC1, else straight
    m = tx.dds_header(2, 64, 64, mip_levels=7)
    flags, mips = struct.unpack_from("<I", m, 8)[0], struct.unpack_from("<I", m, 28)[0]
    assert flags & 0x20000 and mips == 7
    assert struct.unpack_from("<I", m, 4 + 104)[0] == 0x1000 | 0x8 | 0x400000


def test_parse_round_trip_and_legacy(tx):
    for fmt in range(5):
        f, w, h, m, off = tx.dds_parse(tx.dds_header(fmt, 33, 17, 3))
        assert (int(f), w, h, m, off) == (fmt, 33, 17, 3, 148)
    legacy = bytearray(128)
    struct.pack_into("<4s7I", legacy, 0, b"DDS ", 124, 0x1007, 8, 12, 48, 0, 0)
    struct.pack_into("<3I", legacy, 4 + 72, 32, 0x4, struct.unpack("<I", b"DXT5")[0])
    f, w, h, m, off = tx.dds_parse(bytes(legacy))
    assert (int(f), w, h, off) == (2, 12, 8, 128)
    struct.pack_into("<I", legacy, 4 + 80, struct.unpack("<I", b"ATI2")[0])
    with pytest.raises(tx.TexpressoError) as e:
        tx.dds_parse(bytes(legacy))
    assert e.value.status == -1


def test_parse_rejects_what_the_cli_rejects(tx):
    h = bytearray(tx.dds_header(0, 4, 4))
    struct.pack_into("<I", h, 128, 71)          # BC1_UNORM (not sRGB): unsupported by the CLI
    with pytest.raises(tx.TexpressoError):
        tx.dds_parse(bytes(h))
    h = bytearray(tx.dds_header(0, 4, 4))
    struct.pack_into("<I", h, 132, 4)           # Texture3D
    with pytest.raises(tx.TexpressoError):
        tx.dds_parse(bytes(h))
    with pytest.raises(tx.TexpressoError):
        tx.dds_parse(b"DDS " + bytes(10))
    with pytest.raises(tx.TexpressoError):
        tx.dds_header(7, 4, 4)


def test_file_round_trip(tx, tmp_path):
    blocks = np.arange(tx.Format.Bc3.compressed_size(20, 12), dtype=np.uint8)
    p = str(tmp_path / "t.dds")
    tx.write_dds(p, tx.Format.Bc3, 20, 12, blocks)
    f, w, h, m, data = tx.read_dds(p)
    assert (f, w, h, m) == (tx.Format.Bc3, 20, 12, 0)
    assert data == blocks.tobytes()
