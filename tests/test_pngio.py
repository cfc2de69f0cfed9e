"""PNG ingest/output (texpresso_gb300.pngio) against the expansion rules of
cli/src/image/png.rs:30-82 (png crate EXPAND | STRIP_16, then RGBA8)."""
import struct
import zlib

import numpy as np
import pytest

ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


def _filter_rows(rows, bpp, rng):
    """Apply a random PNG filter to each row (the encoder side of the spec)."""
    out, prev = [], np.zeros(rows.shape[1], np.int32)
    for r in rows.astype(np.int32):
        ft = int(rng.integers(0, 5))
        f = np.zeros_like(r)
        for x in range(len(r)):
            a = r[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if ft == 0:
                pred = 0
            elif ft == 1:
                pred = a
            elif ft == 2:
                pred = b
            elif ft == 3:
                pred = (a + b) >> 1
            else:
                p = a + b - c
                pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            f[x] = (r[x] - pred) & 0xFF
        out.append(bytes([ft]) + f.astype(np.uint8).tobytes())
        prev = r
    return b"".join(out)


def _pack(samples, depth):
    h, w, n = samples.shape
    if depth == 8:
        return samples.astype(np.uint8).reshape(h, w * n)
    if depth == 16:
        s = samples.astype(np.uint16).reshape(h, w * n)
        return np.stack([s >> 8, s & 0xFF], axis=2).astype(np.uint8).reshape(h, w * n * 2)
    bits = ((samples.reshape(h, w * n, 1) >> np.arange(depth - 1, -1, -1)) & 1).astype(np.uint8)
    return np.packbits(bits.reshape(h, -1), axis=1)


def _png(samples, depth, ctype, plte=None, trns=None, interlace=False, seed=0):
    rng = np.random.default_rng(seed)
    h, w, n = samples.shape
    bpp = max(1, n * depth // 8)
    if not interlace:
        raw = _filter_rows(_pack(samples, depth), bpp, rng)
    else:
        raw = b""
        for x0, y0, dx, dy in ADAM7:
            sub = samples[y0::dy, x0::dx]
            if sub.size:
                raw += _filter_rows(_pack(sub, depth), bpp, rng)
    ch = lambda k, b: struct.pack(">I", len(b)) + k + b + struct.pack(">I", zlib.crc32(k + b) & 0xFFFFFFFF)
    out = b"\x89PNG\r\n\x1a\n" + ch(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 1 if interlace else 0))
    if plte is not None:
        out += ch(b"PLTE", plte.astype(np.uint8).tobytes())
    if trns is not None:
        out += ch(b"tRNS", trns)
    return out + ch(b"IDAT", zlib.compress(raw)) + ch(b"IEND", b"")


def test_rgba8_round_trip(tx, tmp_path):
    from texpresso_gb300 import pngio
    img = np.random.default_rng(1).integers(0, 256, size=(13, 21, 4), dtype=np.uint8)
    p = str(tmp_path / "x.png")
    pngio.write_png(p, 21, 13, img)
    w, h, out = pngio.read_png(p)
    assert (w, h) == (21, 13) and np.array_equal(out, img)


@pytest.mark.parametrize("interlace", [False, True])
def test_colour_types_and_depths(tx, interlace):
    from texpresso_gb300 import pngio
    rng = np.random.default_rng(2)
    h, w = 11, 17
    # grey 8
    g = rng.integers(0, 256, size=(h, w, 1))
    _, _, o = pngio.read_png(_png(g, 8, 0, interlace=interlace, seed=3))
    assert np.array_equal(o[..., 0], g[..., 0]) and np.all(o[..., 1] == o[..., 0]) and np.all(o[..., 3] == 255)
    # grey+alpha 16 -> high bytes
    ga = rng.integers(0, 65536, size=(h, w, 2))
    _, _, o = pngio.read_png(_png(ga, 16, 4, interlace=interlace, seed=4))
    assert np.array_equal(o[..., 2], ga[..., 0] >> 8) and np.array_equal(o[..., 3], ga[..., 1] >> 8)
    # rgb 8 with a tRNS colour key
    rgb = rng.integers(0, 4, size=(h, w, 3))
    key = struct.pack(">HHH", 1, 2, 3)
    _, _, o = pngio.read_png(_png(rgb, 8, 2, trns=key, interlace=interlace, seed=5))
    hit = np.all(rgb == [1, 2, 3], axis=2)
    assert np.array_equal(o[..., :3], rgb) and np.array_equal(o[..., 3], np.where(hit, 0, 255))
    # 4-bit palette with partial tRNS
    idx = rng.integers(0, 12, size=(h, w, 1))
    plte = rng.integers(0, 256, size=(12, 3))
    trns = bytes([0, 128, 7])
    _, _, o = pngio.read_png(_png(idx, 4, 3, plte=plte, trns=trns, interlace=interlace, seed=6))
    alpha = np.full(12, 255)
    alpha[:3] = [0, 128, 7]
    assert np.array_equal(o[..., :3], plte[idx[..., 0]]) and np.array_equal(o[..., 3], alpha[idx[..., 0]])
    # 2-bit grey scales by 85
    g2 = rng.integers(0, 4, size=(h, w, 1))
    _, _, o = pngio.read_png(_png(g2, 2, 0, interlace=interlace, seed=7))
    assert np.array_equal(o[..., 0], g2[..., 0] * 85)
    # 16-bit rgba
    c16 = rng.integers(0, 65536, size=(h, w, 4))
    _, _, o = pngio.read_png(_png(c16, 16, 6, interlace=interlace, seed=8))
    assert np.array_equal(o, (c16 >> 8).astype(np.uint8))


def test_not_a_png(tx):
    from texpresso_gb300 import pngio
    with pytest.raises(pngio.PngError):
        pngio.read_png(b"GIF89a" + bytes(20))
