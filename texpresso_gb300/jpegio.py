"""JPEG ingest for the CLI-equivalent flow (host side).

read_jpeg mirrors cli/src/image/jpeg.rs:29-57: the file is decoded, and the
CLI widens the decoder's pixel format to RGBA8 (L8 g -> g,g,g,255; RGB24
r,g,b -> r,g,b,255) and rejects every other format (CMYK).

This is an independent decoder written against ITU-T T.81 (JPEG) and JFIF
with numpy; it is not on the GPU path.  It decodes baseline, extended
sequential and progressive Huffman JPEG with 8-bit samples (T.81 Annex G:
spectral selection, successive approximation, end-of-band runs): one or three
components, any sampling factors, interleaved or single-component scans,
restart intervals.  Lossless, hierarchical and arithmetic-coded files raise
JpegError.  The reference's decoder crate (jpeg-decoder 0.3) is not vendored,
so its exact IDCT and upsampling rounding are not reproduced bit for bit:
here the inverse DCT is the exact separable cosine transform in float64,
chroma is upsampled with the triangle ("fancy") filter for 2x1 and 2x2
subsampling and by replication otherwise, and YCbCr -> RGB follows JFIF,
each rounded to nearest and clamped to 0..255.
"""
import math
import struct

import numpy as np


class JpegError(ValueError):
    pass


# zig-zag position k -> natural (row-major) index
ZIGZAG = np.array([
    0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5,
    12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14, 21, 28,
    35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
    58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63], np.int64)

_ZZ = ZIGZAG.tolist()

# C[u, x] = c(u)/2 cos((2x+1) u pi / 16): f = C^T F C is the 8x8 inverse DCT
_C = np.array([[(math.sqrt(0.5) if u == 0 else 1.0) * 0.5 * math.cos((2 * x + 1) * u * math.pi / 16)
                for x in range(8)] for u in range(8)])


class _Huffman:
    """Canonical Huffman table (T.81 Annex C) with a 16-bit lookup: the next
    16 bits index (symbol << 8 | code length); length 0 marks no code."""

    def __init__(self, counts, symbols):
        fast = [0] * 65536
        code, k = 0, 0
        for length in range(1, 17):
            for _ in range(counts[length - 1]):
                lo = code << (16 - length)
                fast[lo:lo + (1 << (16 - length))] = [(symbols[k] << 8) | length] * (1 << (16 - length))
                code += 1
                k += 1
            code <<= 1
        self.fast = fast


class _Bits:
    """Entropy-coded segment reader.  The segment is cut at its RSTn markers
    into intervals with the byte stuffing (FF 00) removed; bits past an
    interval's end read as zero (T.81 F.2.2.5)."""

    def __init__(self, data, pos):
        chunks, cur, n = [], [], len(data)
        while True:
            f = data.find(b"\xff", pos)
            if f < 0 or f + 1 >= n:
                cur.append(data[pos:])
                break
            cur.append(data[pos:f])
            nxt = data[f + 1]
            if nxt == 0x00:
                cur.append(b"\xff")
                pos = f + 2
            elif 0xD0 <= nxt <= 0xD7:
                chunks.append(b"".join(cur))
                cur = []
                pos = f + 2
            elif nxt == 0xFF:
                pos = f + 1  # fill byte
            else:
                break  # another marker ends the segment
        chunks.append(b"".join(cur))
        self.chunks, self.ci = chunks, 0
        self._start(chunks[0])

    def _start(self, chunk):
        self.buf, self.pos, self.end = chunk, 0, len(chunk)
        self.acc, self.n = 0, 0

    def _fill(self, need):
        while self.n < need:
            b = self.buf[self.pos:self.pos + 8]
            if self.pos + 8 > self.end:
                b = b + bytes(8 - len(b))  # past the end: zero bits
            self.pos += 8
            self.acc = (self.acc << 64) | int.from_bytes(b, "big")
            self.n += 64

    def bit(self):
        if self.n < 1:
            self._fill(1)
        self.n -= 1
        v = (self.acc >> self.n) & 1
        self.acc &= (1 << self.n) - 1
        return v

    def bits(self, k):
        if k == 0:
            return 0
        if self.n < k:
            self._fill(k)
        self.n -= k
        v = self.acc >> self.n
        self.acc &= (1 << self.n) - 1
        return v

    def decode(self, table):
        if self.n < 16:
            self._fill(16)
        e = table.fast[(self.acc >> (self.n - 16)) & 0xFFFF]
        length = e & 0xFF
        if length == 0:
            raise JpegError("bad Huffman code")
        self.n -= length
        self.acc &= (1 << self.n) - 1
        return e >> 8

    def restart(self):
        """Move to the interval after the next RSTn marker."""
        self.ci += 1
        if self.ci >= len(self.chunks):
            raise JpegError("missing restart marker")
        self._start(self.chunks[self.ci])


def _extend(v, s):
    """T.81 F.2.2.1 EXTEND: s-bit magnitude category to a signed value."""
    return v - (1 << s) + 1 if s and v < (1 << (s - 1)) else v


def _parse(data):
    if data[:2] != b"\xff\xd8":
        raise JpegError("not a JPEG file (no SOI marker)")
    pos = 2
    qt, dc, ac = {}, {}, {}
    frame, restart, adobe = None, 0, None
    scans = []
    while pos < len(data):
        if data[pos] != 0xFF:
            raise JpegError("marker expected at byte %d" % pos)
        m = data[pos + 1]
        pos += 2
        if m == 0xFF:  # fill byte
            pos -= 1
            continue
        if m == 0xD9:  # EOI
            break
        if 0xD0 <= m <= 0xD7 or m == 0x01:
            continue
        (seg_len,) = struct.unpack(">H", data[pos:pos + 2])
        seg = data[pos + 2:pos + seg_len]
        pos += seg_len
        if m == 0xDB:  # DQT
            i = 0
            while i < len(seg):
                pq, tq = seg[i] >> 4, seg[i] & 15
                if pq == 0:
                    q = np.frombuffer(seg, np.uint8, 64, i + 1).astype(np.int64)
                    i += 65
                else:
                    q = np.frombuffer(seg, ">u2", 64, i + 1).astype(np.int64)
                    i += 129
                qt[tq] = q  # zig-zag order
        elif m == 0xC4:  # DHT
            i = 0
            while i < len(seg):
                tc, th = seg[i] >> 4, seg[i] & 15
                counts = list(seg[i + 1:i + 17])
                n = sum(counts)
                (dc if tc == 0 else ac)[th] = _Huffman(counts, list(seg[i + 17:i + 17 + n]))
                i += 17 + n
        elif m in (0xC0, 0xC1, 0xC2):  # SOF0 baseline, SOF1 extended sequential, SOF2 progressive
            p, h, w, nf = struct.unpack(">BHHB", seg[:6])
            if p != 8:
                raise JpegError("%d-bit samples are not supported" % p)
            comps = []
            for k in range(nf):
                cid, hv, tq = seg[6 + 3 * k], seg[7 + 3 * k], seg[8 + 3 * k]
                comps.append({"id": cid, "h": hv >> 4, "v": hv & 15, "tq": tq})
            frame = {"w": w, "h": h, "comps": comps, "progressive": m == 0xC2}
        elif 0xC3 <= m <= 0xCF and m not in (0xC4, 0xC8, 0xCC):
            raise JpegError("SOF%d (lossless, hierarchical or arithmetic) is not supported" % (m - 0xC0))
        elif m == 0xDD:  # DRI
            (restart,) = struct.unpack(">H", seg[:2])
        elif m == 0xEE and seg[:5] == b"Adobe" and len(seg) >= 12:
            adobe = seg[11]  # colour transform: 0 none (RGB/CMYK), 1 YCbCr, 2 YCCK
        elif m == 0xDA:  # SOS: the entropy-coded data follows
            if frame is None:
                raise JpegError("scan before frame header")
            ns = seg[0]
            sc = [(seg[1 + 2 * k], seg[2 + 2 * k] >> 4, seg[2 + 2 * k] & 15) for k in range(ns)]
            ss, se, ah, al = seg[1 + 2 * ns], seg[2 + 2 * ns], seg[3 + 2 * ns] >> 4, seg[3 + 2 * ns] & 15
            if not frame["progressive"] and (ss, se, ah, al) != (0, 63, 0, 0):
                raise JpegError("spectral selection / successive approximation in a sequential scan")
            if frame["progressive"] and (se < ss or se > 63 or (ss == 0) != (se == 0) or (ss > 0 and ns != 1)):
                raise JpegError("invalid progressive scan parameters")
            scans.append((sc, pos, restart, dict(dc), dict(ac), (ss, se, ah, al)))
            # skip the entropy-coded segment: to the next marker that is not RSTn or stuffing
            while True:
                pos = data.find(b"\xff", pos)
                if pos < 0 or pos + 1 >= len(data):
                    pos = len(data)
                    break
                nxt = data[pos + 1]
                if nxt != 0x00 and nxt != 0xFF and not 0xD0 <= nxt <= 0xD7:
                    break
                pos += 1
    if frame is None:
        raise JpegError("no frame header")
    return frame, qt, scans, adobe


def _decode_coefficients(data, frame, scans):
    comps = frame["comps"]
    hmax = max(c["h"] for c in comps)
    vmax = max(c["v"] for c in comps)
    mcux = -(-frame["w"] // (8 * hmax))
    mcuy = -(-frame["h"] // (8 * vmax))
    for c in comps:
        # blocks allocated for the interleaved MCU grid (covers the component's own extent)
        c["bw"], c["bh"] = mcux * c["h"], mcuy * c["v"]
        c["coef"] = [0] * (c["bh"] * c["bw"] * 64)  # flat (block row, block, natural order)
        # extent of a single-component scan (T.81 A.2.2)
        c["cw"] = -(-(-(-frame["w"] * c["h"] // hmax)) // 8)
        c["ch"] = -(-(-(-frame["h"] * c["v"] // vmax)) // 8)
    byid = {c["id"]: c for c in comps}
    for sc, pos, restart, dct, act, (ss, se, ah, al) in scans:
        sel = []
        for cid, td, ta in sc:
            if cid not in byid:
                raise JpegError("scan names an unknown component")
            # a progressive DC scan uses no AC table, an AC scan no DC table
            need_dc, need_ac = ss == 0 and ah == 0, se > 0
            if (need_dc and td not in dct) or (need_ac and ta not in act):
                raise JpegError("scan uses an undefined Huffman table")
            sel.append((byid[cid], dct.get(td), act.get(ta)))
        bits = _Bits(data, pos)
        pred = [0] * len(sel)
        if len(sel) == 1:
            c = sel[0][0]
            units = [[(0, by, bx)] for by in range(c["ch"]) for bx in range(c["cw"])]
        else:
            units = []
            for my in range(mcuy):
                for mx in range(mcux):
                    u = []
                    for k, (c, _, _) in enumerate(sel):
                        for v in range(c["v"]):
                            for h in range(c["h"]):
                                u.append((k, my * c["v"] + v, mx * c["h"] + h))
                    units.append(u)
        eobrun = [0]
        for n, unit in enumerate(units):
            if restart and n and n % restart == 0:
                bits.restart()
                pred = [0] * len(sel)
                eobrun[0] = 0
            for k, by, bx in unit:
                c, dt, at = sel[k]
                coef = c["coef"]
                b0 = (by * c["bw"] + bx) * 64
                if frame["progressive"]:
                    if ss == 0:
                        if ah == 0:  # DC first scan: the difference, scaled by 2^Al (G.1.2.1)
                            s = bits.decode(dt)
                            pred[k] += _extend(bits.bits(s), s)
                            coef[b0] = pred[k] << al
                        elif bits.bit():  # DC refinement: one more bit
                            coef[b0] |= 1 << al
                    elif ah == 0:
                        _ac_first(bits, at, coef, b0, ss, se, al, eobrun)
                    else:
                        _ac_refine(bits, at, coef, b0, ss, se, al, eobrun)
                    continue
                s = bits.decode(dt)
                pred[k] += _extend(bits.bits(s), s)
                coef[b0] = pred[k]
                z = 1
                while z < 64:
                    rs = bits.decode(at)
                    r, s = rs >> 4, rs & 15
                    if s == 0:
                        if r != 15:
                            break  # EOB
                        z += 16
                        continue
                    z += r
                    if z > 63:
                        raise JpegError("coefficient index out of range")
                    v = bits.bits(s)
                    coef[b0 + _ZZ[z]] = v if v >> (s - 1) else v - (1 << s) + 1
                    z += 1
    for c in comps:
        c["coef"] = np.array(c["coef"], np.int64).reshape(c["bh"], c["bw"], 64)
    return comps, hmax, vmax


def _ac_first(bits, table, coef, b0, ss, se, al, eobrun):
    """First AC scan of one block (T.81 G.1.2.2): run/size symbols scaled by
    2^Al, ZRL, and end-of-band runs that cover whole blocks."""
    if eobrun[0] > 0:
        eobrun[0] -= 1
        return
    k = ss
    while k <= se:
        rs = bits.decode(table)
        r, s = rs >> 4, rs & 15
        if s:
            k += r
            if k > se:
                raise JpegError("coefficient index out of range")
            coef[b0 + _ZZ[k]] = _extend(bits.bits(s), s) << al
            k += 1
        elif r == 15:
            k += 16
        else:
            eobrun[0] = (1 << r) - 1 + (bits.bits(r) if r else 0)
            return


def _ac_refine(bits, table, coef, b0, ss, se, al, eobrun):
    """AC refinement scan of one block (T.81 G.1.2.3): a correction bit for
    every coefficient already non-zero, new coefficients of magnitude 2^Al
    placed after runs of zero-history coefficients, and end-of-band runs
    during which only correction bits arrive."""
    p1, m1 = 1 << al, -1 << al
    k = ss
    if eobrun[0] == 0:
        while k <= se:
            rs = bits.decode(table)
            r, s = rs >> 4, rs & 15
            if s:
                if s != 1:
                    raise JpegError("bad refinement symbol")
                s = p1 if bits.bit() else m1
            elif r != 15:
                eobrun[0] = (1 << r) + (bits.bits(r) if r else 0)
                break
            while k <= se:
                z = b0 + _ZZ[k]
                if coef[z] != 0:
                    if bits.bit() and (coef[z] & p1) == 0:
                        coef[z] += p1 if coef[z] >= 0 else m1
                else:
                    r -= 1
                    if r < 0:
                        break
                k += 1
            if s and k <= se:
                coef[b0 + _ZZ[k]] = s
            k += 1
    if eobrun[0] > 0:
        while k <= se:
            z = b0 + _ZZ[k]
            if coef[z] != 0 and bits.bit() and (coef[z] & p1) == 0:
                coef[z] += p1 if coef[z] >= 0 else m1
            k += 1
        eobrun[0] -= 1


def _idct_plane(c, q):
    """Dequantise and inverse-DCT every block of a component: samples 0..255."""
    qn = np.zeros(64, np.int64)
    qn[ZIGZAG] = q
    f = (c["coef"] * qn).reshape(c["bh"], c["bw"], 8, 8).astype(np.float64)
    px = np.matmul(np.matmul(_C.T, f), _C) + 128.0  # per block: C^T F C
    px = np.clip(np.floor(px + 0.5), 0, 255)
    return px.transpose(0, 2, 1, 3).reshape(c["bh"] * 8, c["bw"] * 8)


def _upsample(p, fx, fy, w, h):
    """Component plane to full resolution: triangle filter for 2x1 / 2x2, else replication."""
    if fx == 1 and fy == 1:
        return p[:h, :w]
    if (fx, fy) in ((2, 1), (2, 2)):
        # each output sample weighs its own input sample 3/4 and the nearer
        # neighbour 1/4 in each subsampled direction, edges replicated
        q = p.astype(np.int64)
        if fy == 2:
            up = np.vstack([q[:1], q[:-1]])
            dn = np.vstack([q[1:], q[-1:]])
            rows = np.empty((2 * q.shape[0], q.shape[1]), np.int64)
            rows[0::2] = 3 * q + up   # 4x scale, vertical triangle
            rows[1::2] = 3 * q + dn
            lf = np.hstack([rows[:, :1], rows[:, :-1]])
            rt = np.hstack([rows[:, 1:], rows[:, -1:]])
            out = np.empty((rows.shape[0], 2 * rows.shape[1]), np.int64)
            out[:, 0::2] = (3 * rows + lf + 8) >> 4
            out[:, 1::2] = (3 * rows + rt + 7) >> 4
        else:
            lf = np.hstack([q[:, :1], q[:, :-1]])
            rt = np.hstack([q[:, 1:], q[:, -1:]])
            out = np.empty((q.shape[0], 2 * q.shape[1]), np.int64)
            out[:, 0::2] = (3 * q + lf + 1) >> 2
            out[:, 1::2] = (3 * q + rt + 2) >> 2
        return out[:h, :w].astype(np.float64)
    return np.repeat(np.repeat(p, fy, axis=0), fx, axis=1)[:h, :w]


def decode_jpeg(data):
    """Decode JPEG bytes to (pixels uint8 (h, w, channels), channels) with
    channels 1 (grey) or 3 (RGB)."""
    data = bytes(data)
    frame, qt, scans, adobe = _parse(data)
    comps, hmax, vmax = _decode_coefficients(data, frame, scans)
    w, h = frame["w"], frame["h"]
    if len(comps) not in (1, 3):
        raise JpegError("JPEG files with %d components (CMYK) are not supported" % len(comps))
    planes = []
    for c in comps:
        if c["tq"] not in qt:
            raise JpegError("undefined quantisation table")
        p = _idct_plane(c, qt[c["tq"]])
        # the component's own extent (T.81 A.1.1): filters replicate its edge
        # samples, never the block padding beyond it
        p = p[:-(-h * c["v"] // vmax), :-(-w * c["h"] // hmax)]
        planes.append(_upsample(p, hmax // c["h"], vmax // c["v"], w, h))
    if len(comps) == 1:
        return planes[0].astype(np.uint8)[:, :, None], 1
    y, cb, cr = planes
    if adobe == 0:  # stored as RGB
        rgb = np.stack([y, cb, cr], axis=-1)
    else:
        r = y + 1.402 * (cr - 128.0)
        g = y - 0.344136 * (cb - 128.0) - 0.714136 * (cr - 128.0)
        b = y + 1.772 * (cb - 128.0)
        rgb = np.stack([r, g, b], axis=-1)
    return np.clip(np.floor(rgb + 0.5), 0, 255).astype(np.uint8), 3


def read_jpeg(path_or_bytes):
    """cli/src/image/jpeg.rs:29-57: (width, height, RGBA8 array (h, w, 4)) of a JPEG file."""
    if isinstance(path_or_bytes, (bytes, bytearray, memoryview)):
        data = bytes(path_or_bytes)
    else:
        with open(path_or_bytes, "rb") as f:
            data = f.read()
    px, ch = decode_jpeg(data)
    h, w = px.shape[:2]
    rgba = np.empty((h, w, 4), np.uint8)
    rgba[..., :3] = px if ch == 3 else px[..., :1]
    rgba[..., 3] = 255
    return w, h, rgba
