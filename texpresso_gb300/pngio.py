"""PNG ingest and output for the CLI-equivalent flow (host side).

read_png mirrors cli/src/image/png.rs:30-70: the png crate decodes with
Transformations::EXPAND | STRIP_16 (palette -> RGB, tRNS -> alpha, bit depths
below 8 scaled up to 8, 16-bit samples reduced to their high byte) and the
CLI then widens every colour type to RGBA8 (grey g -> g,g,g,255; grey+alpha
-> g,g,g,a; RGB -> r,g,b,255).  write_png mirrors png.rs:72-82: one RGBA8
image, 8 bits per sample.  Interlaced (Adam7) files are de-interlaced.

This is an independent decoder written against the PNG specification with
zlib and numpy; it is not on the GPU path.
"""
import struct
import zlib

import numpy as np

_SIG = b"\x89PNG\r\n\x1a\n"
_CHANNELS = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}
_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


class PngError(ValueError):
    pass


def _unfilter(raw, rows, stride, bpp):
    """Undo the per-row filters (PNG spec section 9) of `rows` rows."""
    out = np.zeros((rows, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    pos = 0
    for y in range(rows):
        ft = raw[pos]
        line = np.frombuffer(raw, np.uint8, stride, pos + 1).astype(np.int32)
        pos += 1 + stride
        if ft == 0:
            cur = line
        elif ft == 2:
            cur = (line + prev) & 0xFF
        elif ft in (1, 3, 4):
            cur = np.zeros(stride, np.int32)
            for x in range(stride):
                a = cur[x - bpp] if x >= bpp else 0
                if ft == 1:
                    pred = a
                elif ft == 3:
                    pred = (a + prev[x]) >> 1
                else:
                    b, c = prev[x], (prev[x - bpp] if x >= bpp else 0)
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + pred) & 0xFF
        else:
            raise PngError("bad filter type %d" % ft)
        out[y] = cur
        prev = cur
    return out, pos


def _samples(rows, width, depth, nch):
    """Unpack filtered-away rows into (h, w, nch) sample values."""
    if depth == 8:
        return rows[:, :width * nch].reshape(rows.shape[0], width, nch).astype(np.uint16)
    if depth == 16:
        v = rows[:, :width * nch * 2].reshape(rows.shape[0], width * nch, 2).astype(np.uint16)
        return ((v[..., 0] << 8) | v[..., 1]).reshape(rows.shape[0], width, nch)
    bits = np.unpackbits(rows, axis=1)[:, :width * nch * depth].reshape(rows.shape[0], width * nch, depth)
    weights = (1 << np.arange(depth - 1, -1, -1)).astype(np.uint16)
    return (bits.astype(np.uint16) * weights).sum(axis=2).astype(np.uint16).reshape(rows.shape[0], width, nch)


def read_png(path_or_bytes):
    """(width, height, RGBA8 array (h, w, 4)) of a PNG file."""
    data = path_or_bytes if isinstance(path_or_bytes, (bytes, bytearray)) else open(path_or_bytes, "rb").read()
    if data[:8] != _SIG:
        raise PngError("not a PNG file")
    pos, idat, plte, trns, hdr = 8, [], None, None, None
    while pos + 8 <= len(data):
        n, kind = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            plte = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if hdr is None:
        raise PngError("missing IHDR")
    width, height, depth, ctype, _, _, interlace = hdr
    if ctype not in _CHANNELS:
        raise PngError("bad colour type %d" % ctype)
    nch = _CHANNELS[ctype]
    raw = zlib.decompress(b"".join(idat))
    bpp = max(1, nch * depth // 8)
    samples = np.zeros((height, width, nch), np.uint16)
    if interlace == 0:
        stride = (width * nch * depth + 7) // 8
        rows, _ = _unfilter(raw, height, stride, bpp)
        samples = _samples(rows, width, depth, nch)
    else:
        pos = 0
        for x0, y0, dx, dy in _ADAM7:
            pw, ph = (width - x0 + dx - 1) // dx, (height - y0 + dy - 1) // dy
            if pw <= 0 or ph <= 0:
                continue
            stride = (pw * nch * depth + 7) // 8
            rows, used = _unfilter(raw[pos:], ph, stride, bpp)
            pos += used
            samples[y0::dy, x0::dx] = _samples(rows, pw, depth, nch)
    # EXPAND: palette -> RGB(A); tRNS -> alpha; low bit depths -> 8 bits
    alpha = None
    if ctype == 3:
        idx = samples[..., 0].astype(np.intp)
        rgb = plte[np.minimum(idx, len(plte) - 1)].astype(np.uint16)
        if trns is not None:
            t = np.full(256, 255, np.uint16)
            t[:len(trns)] = np.frombuffer(trns, np.uint8)
            alpha = t[idx]
        samples, ctype, depth = rgb, 2, 8
    elif trns is not None and ctype in (0, 2):
        key = struct.unpack(">H", trns[:2])[0] if ctype == 0 else struct.unpack(">HHH", trns[:6])
        match = samples[..., 0] == key if ctype == 0 else np.all(samples == np.array(key, np.uint16), axis=2)
        alpha = np.where(match, 0, (1 << depth) - 1).astype(np.uint16)
    if depth == 16:  # STRIP_16: keep the high byte
        samples = samples >> 8
        alpha = None if alpha is None else alpha >> 8
    elif depth < 8:  # scale 1/2/4-bit grey up to 8 bits
        scale = 255 // ((1 << depth) - 1)
        samples = samples * scale
        alpha = None if alpha is None else np.where(alpha > 0, 255, 0)
    s = samples.astype(np.uint8)
    out = np.empty((height, width, 4), np.uint8)
    if ctype in (0, 4):          # grey (+alpha): g, g, g, a
        out[..., 0] = out[..., 1] = out[..., 2] = s[..., 0]
        out[..., 3] = s[..., 1] if ctype == 4 else 255
    else:                        # rgb (+alpha)
        out[..., :3] = s[..., :3]
        out[..., 3] = s[..., 3] if ctype == 6 else 255
    if alpha is not None:
        out[..., 3] = alpha.astype(np.uint8)
    return width, height, out


def _chunk(kind, body):
    return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)


def write_png(path, width, height, rgba):
    """Write RGBA8 pixels as an 8-bit RGBA PNG (unfiltered rows)."""
    px = np.ascontiguousarray(rgba, dtype=np.uint8).reshape(height, width * 4)
    raw = np.concatenate([np.zeros((height, 1), np.uint8), px], axis=1).tobytes()
    data = (_SIG + _chunk(b"IHDR", struct.pack(">IIBBBBB", width, height, 8, 6, 0, 0, 0)) +
            _chunk(b"IDAT", zlib.compress(raw, 6)) + _chunk(b"IEND", b""))
    with open(path, "wb") as f:
        f.write(data)
