"""JPEG ingest (texpresso_gb300/jpegio.py, cli/src/image/jpeg.rs:29-57).

The image has no JPEG encoder, so this file holds a small baseline encoder
written against ITU-T T.81 (forward DCT, quantisation, canonical Huffman
tables of uniform code length, byte stuffing, restart markers).  Files it
writes must decode back to the source within the quantisation error, in
every layout the decoder supports: grey, 4:4:4, 4:2:2, 4:2:0, interleaved
and one-component scans, restart intervals, odd sizes.  The CLI's widening
to RGBA8 and its refusal of CMYK and progressive files are checked too."""
import struct

import numpy as np
import pytest

from texpresso_gb300 import jpegio

C = jpegio._C


class _BitWriter:
    def __init__(self):
        self.out = bytearray()
        self.acc, self.n = 0, 0

    def put(self, v, n):
        for i in range(n - 1, -1, -1):
            self.acc = (self.acc << 1) | ((v >> i) & 1)
            self.n += 1
            if self.n == 8:
                self.out.append(self.acc)
                if self.acc == 0xFF:
                    self.out.append(0)  # byte stuffing
                self.acc, self.n = 0, 0

    def flush(self):
        if self.n:
            self.put((1 << (8 - self.n)) - 1, 8 - self.n)  # pad with 1-bits


def _uniform_table(symbols, length):
    counts = [0] * 16
    counts[length - 1] = len(symbols)
    codes = {s: (i, length) for i, s in enumerate(symbols)}
    return counts, list(symbols), codes


DC_SYMS = list(range(12))
# run/size symbols, ZRL, and the end-of-band runs EOB0..EOB14 of progressive scans
AC_SYMS = [0x00, 0xF0] + [(r << 4) | s for r in range(16) for s in range(1, 11)] + [r << 4 for r in range(1, 15)]
DC_TAB = _uniform_table(DC_SYMS, 4)
AC_TAB = _uniform_table(AC_SYMS, 8)


def _category(v):
    return int(abs(v)).bit_length()


def _encode_block(bw, coef_zz, pred):
    dc = int(coef_zz[0])
    d = dc - pred
    s = _category(d)
    code, ln = DC_TAB[2][s]
    bw.put(code, ln)
    if s:
        bw.put(d if d > 0 else d + (1 << s) - 1, s)
    run = 0
    last = max([k for k in range(1, 64) if coef_zz[k] != 0], default=0)
    for k in range(1, last + 1):
        v = int(coef_zz[k])
        if v == 0:
            run += 1
            continue
        while run > 15:
            code, ln = AC_TAB[2][0xF0]
            bw.put(code, ln)
            run -= 16
        s = _category(v)
        code, ln = AC_TAB[2][(run << 4) | s]
        bw.put(code, ln)
        bw.put(v if v > 0 else v + (1 << s) - 1, s)
        run = 0
    if last < 63:
        code, ln = AC_TAB[2][0x00]
        bw.put(code, ln)
    return dc


def _blocks(plane, q):
    """Quantised zig-zag coefficients of every 8x8 block of a padded plane."""
    h, w = plane.shape
    f = plane.reshape(h // 8, 8, w // 8, 8).transpose(0, 2, 1, 3) - 128.0
    F = np.einsum("ux,abxy,vy->abuv", C, f, C).reshape(h // 8, w // 8, 64)
    qn = np.zeros(64)
    qn[jpegio.ZIGZAG] = q
    return np.round(F / qn)[:, :, jpegio.ZIGZAG].astype(np.int64)


def _pad(p, h, w):
    return np.pad(p, ((0, h - p.shape[0]), (0, w - p.shape[1])), mode="edge")


def encode(img, hv=(1, 1), restart=0, separate_scans=False, q=None, progressive=None):
    """Baseline JPEG of img (h, w) grey or (h, w, 3) RGB; hv = luma sampling
    factors (chroma 1x1).  progressive: a list of (Ss, Se, Ah, Al) scans, DC
    scans interleaved over all components, AC scans one per component."""
    img = np.asarray(img)
    h, w = img.shape[:2]
    q = np.full(64, 2, np.int64) if q is None else q
    if img.ndim == 2:
        planes = [img.astype(np.float64)]
        factors = [(1, 1)]
    else:
        r, g, b = (img[..., i].astype(np.float64) for i in range(3))
        y = 0.299 * r + 0.587 * g + 0.114 * b
        cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
        cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128
        planes = [y, cb, cr]
        factors = [hv, (1, 1), (1, 1)]
    hmax, vmax = max(f[0] for f in factors), max(f[1] for f in factors)
    mcux, mcuy = -(-w // (8 * hmax)), -(-h // (8 * vmax))
    comp_blocks, extents = [], []
    for p, (fh, fv) in zip(planes, factors):
        # the component's own extent, then subsampled by box averaging
        ch, cw = -(-h * fv // vmax), -(-w * fh // hmax)
        sx, sy = hmax // fh, vmax // fv
        full = _pad(p, ch * sy, cw * sx)
        sub = full.reshape(ch, sy, cw, sx).mean(axis=(1, 3))
        padded = _pad(sub, mcuy * fv * 8, mcux * fh * 8)
        comp_blocks.append(_blocks(np.clip(np.round(padded), 0, 255), q))
        extents.append((-(-ch // 8), -(-cw // 8)))
    out = bytearray(b"\xff\xd8")
    out += b"\xff\xdb" + struct.pack(">HB", 67, 0) + bytes(q.astype(np.uint8))
    nf = len(planes)
    sof = struct.pack(">BHHB", 8, h, w, nf)
    for k, (fh, fv) in enumerate(factors):
        sof += bytes([k + 1, (fh << 4) | fv, 0])
    out += (b"\xff\xc2" if progressive else b"\xff\xc0") + struct.pack(">H", 2 + len(sof)) + sof
    for tc, tab in ((0, DC_TAB), (1, AC_TAB)):
        body = bytes([tc << 4]) + bytes(tab[0]) + bytes(tab[1])
        out += b"\xff\xc4" + struct.pack(">H", 2 + len(body)) + body
    if restart:
        out += b"\xff\xdd" + struct.pack(">HH", 4, restart)

    def scan(comp_ids):
        sos = bytes([len(comp_ids)])
        for k in comp_ids:
            sos += bytes([k + 1, 0x00])
        sos += bytes([0, 63, 0])
        seg = b"\xff\xda" + struct.pack(">H", 2 + len(sos)) + sos
        bw = _BitWriter()
        pred = {k: 0 for k in comp_ids}
        if len(comp_ids) == 1:
            k = comp_ids[0]
            units = [[(k, by, bx)] for by in range(extents[k][0]) for bx in range(extents[k][1])]
        else:
            units = [[(k, my * factors[k][1] + v, mx * factors[k][0] + u)
                      for k in comp_ids for v in range(factors[k][1]) for u in range(factors[k][0])]
                     for my in range(mcuy) for mx in range(mcux)]
        marker = 0
        for n, unit in enumerate(units):
            if restart and n and n % restart == 0:
                bw.flush()
                bw.out += bytes([0xFF, 0xD0 + marker])
                marker = (marker + 1) & 7
                pred = {k: 0 for k in comp_ids}
            for k, by, bx in unit:
                pred[k] = _encode_block(bw, comp_blocks[k][by, bx], pred[k])
        bw.flush()
        return seg + bytes(bw.out)

    def pscan(comp_ids, ss, se, ah, al):
        sos = bytes([len(comp_ids)])
        for k in comp_ids:
            sos += bytes([k + 1, 0x00])
        sos += bytes([ss, se, (ah << 4) | al])
        seg = b"\xff\xda" + struct.pack(">H", 2 + len(sos)) + sos
        bw = _BitWriter()
        if len(comp_ids) == 1:
            k = comp_ids[0]
            units = [[(k, by, bx)] for by in range(extents[k][0]) for bx in range(extents[k][1])]
        else:
            units = [[(k, my * factors[k][1] + v, mx * factors[k][0] + u)
                      for k in comp_ids for v in range(factors[k][1]) for u in range(factors[k][0])]
                     for my in range(mcuy) for mx in range(mcux)]
        st = {"eobrun": 0, "be": [], "pred": {k: 0 for k in comp_ids}}

        def sym(v):
            code, ln = AC_TAB[2][v]
            bw.put(code, ln)

        def emit_eobrun():
            if st["eobrun"]:
                n = st["eobrun"].bit_length() - 1
                sym(n << 4)
                if n:
                    bw.put(st["eobrun"] & ((1 << n) - 1), n)
                st["eobrun"] = 0
                for b in st["be"]:
                    bw.put(b, 1)
                st["be"] = []

        marker = 0
        for n, unit in enumerate(units):
            if restart and n and n % restart == 0:
                emit_eobrun()
                bw.flush()
                bw.out += bytes([0xFF, 0xD0 + marker])
                marker = (marker + 1) & 7
                st["pred"] = {k: 0 for k in comp_ids}
            for k, by, bx in unit:
                zz = comp_blocks[k][by, bx]
                if ss == 0:
                    if ah == 0:
                        v = int(zz[0]) >> al
                        d = v - st["pred"][k]
                        st["pred"][k] = v
                        c = _category(d)
                        code, ln = DC_TAB[2][c]
                        bw.put(code, ln)
                        if c:
                            bw.put(d if d > 0 else d + (1 << c) - 1, c)
                    else:
                        bw.put((int(zz[0]) >> al) & 1, 1)
                elif ah == 0:  # AC first (T.81 G.1.2.2, as libjpeg's encoder)
                    r = 0
                    for z in range(ss, se + 1):
                        a = abs(int(zz[z])) >> al
                        if a == 0:
                            r += 1
                            continue
                        emit_eobrun()
                        while r > 15:
                            sym(0xF0)
                            r -= 16
                        c = a.bit_length()
                        sym((r << 4) | c)
                        bw.put(a if zz[z] > 0 else (~a) & ((1 << c) - 1), c)
                        r = 0
                    if r:
                        st["eobrun"] += 1
                        if st["eobrun"] == 0x7FFF:
                            emit_eobrun()
                else:  # AC refinement (T.81 G.1.2.3, as libjpeg's encoder)
                    absv = [abs(int(zz[z])) >> al for z in range(64)]
                    eob = max([z for z in range(ss, se + 1) if absv[z] == 1], default=-1)
                    r, br = 0, []
                    for z in range(ss, se + 1):
                        t = absv[z]
                        if t == 0:
                            r += 1
                            continue
                        while r > 15 and z <= eob:
                            emit_eobrun()
                            sym(0xF0)
                            r -= 16
                            for b in br:
                                bw.put(b, 1)
                            br = []
                        if t > 1:
                            br.append(t & 1)
                            continue
                        emit_eobrun()
                        sym((r << 4) | 1)
                        bw.put(0 if zz[z] < 0 else 1, 1)
                        for b in br:
                            bw.put(b, 1)
                        br, r = [], 0
                    if r or br:
                        st["eobrun"] += 1
                        st["be"] += br
                        if st["eobrun"] == 0x7FFF:
                            emit_eobrun()
        emit_eobrun()
        bw.flush()
        return seg + bytes(bw.out)

    if progressive:
        for ss, se, ah, al in progressive:
            if ss == 0:
                out += pscan(list(range(nf)), ss, se, ah, al)
            else:
                for k in range(nf):
                    out += pscan([k], ss, se, ah, al)
    elif separate_scans:
        for k in range(nf):
            out += scan([k])
    else:
        out += scan(list(range(nf)))
    out += b"\xff\xd9"
    return bytes(out)


def _image(h, w, seed):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:h, 0:w]
    base = np.stack([120 + 100 * np.sin(xx / 9.0 + k) * np.cos(yy / 13.0 - k) for k in range(3)], -1)
    return np.clip(base + rng.normal(0, 2, base.shape), 0, 255).astype(np.uint8)


def _ycc_roundtrip(img):
    """RGB through the encoder's forward and the decoder's inverse colour
    transforms at full resolution (the part of the error not due to DCT or
    subsampling)."""
    r, g, b = (img[..., i].astype(np.float64) for i in range(3))
    y = np.round(0.299 * r + 0.587 * g + 0.114 * b)
    cb = np.round(-0.168736 * r - 0.331264 * g + 0.5 * b + 128)
    cr = np.round(0.5 * r - 0.418688 * g - 0.081312 * b + 128)
    out = np.stack([y + 1.402 * (cr - 128), y - 0.344136 * (cb - 128) - 0.714136 * (cr - 128),
                    y + 1.772 * (cb - 128)], -1)
    return np.clip(np.floor(out + 0.5), 0, 255)


@pytest.mark.parametrize("hv", [(1, 1), (2, 1), (2, 2)])
@pytest.mark.parametrize("restart", [0, 3])
def test_colour_roundtrip(hv, restart):
    img = _image(37, 53, seed=hv[0] * 10 + hv[1] + restart)
    w, h, rgba = jpegio.read_jpeg(encode(img, hv=hv, restart=restart))
    assert (w, h) == (53, 37) and rgba.shape == (37, 53, 4)
    assert np.all(rgba[..., 3] == 255)
    err = np.abs(rgba[..., :3].astype(np.int64) - img.astype(np.int64))
    if hv == (1, 1):
        # full-resolution chroma: only quantisation (step 2) and colour rounding
        assert np.abs(rgba[..., :3] - _ycc_roundtrip(img)).max() <= 6
    assert err.mean() < (2.0 if hv == (1, 1) else 6.0), err.mean()


def test_separate_scans_and_odd_sizes():
    img = _image(23, 41, seed=3)
    a = jpegio.read_jpeg(encode(img, hv=(2, 2)))[2]
    b = jpegio.read_jpeg(encode(img, hv=(2, 2), separate_scans=True))[2]
    assert np.array_equal(a, b)  # the same coefficients, interleaved or not


def test_grey_widens_like_the_cli():
    img = _image(19, 30, seed=4)[..., 1]
    w, h, rgba = jpegio.read_jpeg(encode(img, restart=2))
    assert (w, h) == (30, 19)
    assert np.array_equal(rgba[..., 0], rgba[..., 1]) and np.array_equal(rgba[..., 0], rgba[..., 2])
    assert np.all(rgba[..., 3] == 255)
    assert np.abs(rgba[..., 0].astype(np.int64) - img).max() <= 3


def test_exact_coefficients_decode_exactly():
    """A flat block with DC only decodes to its level exactly (IDCT, level
    shift and rounding), in grey and in colour."""
    for level in (0, 37, 128, 200, 255):
        img = np.full((8, 8), level, np.uint8)
        q = np.ones(64, np.int64)
        rgba = jpegio.read_jpeg(encode(img, q=q))[2]
        assert np.all(rgba[..., 0] == level)


PROGRESSIVE = [
    [(0, 0, 0, 0), (1, 63, 0, 0)],                                   # spectral selection only
    [(0, 0, 0, 1), (1, 5, 0, 2), (6, 63, 0, 2), (0, 0, 1, 0),         # libjpeg-like script
     (1, 63, 2, 1), (1, 63, 1, 0)],
    [(0, 0, 0, 2), (0, 0, 2, 1), (0, 0, 1, 0), (1, 2, 0, 0), (3, 63, 0, 3),
     (3, 63, 3, 2), (3, 63, 2, 1), (3, 63, 1, 0)],
]


@pytest.mark.parametrize("script", range(len(PROGRESSIVE)))
@pytest.mark.parametrize("hv,restart", [((1, 1), 0), ((2, 2), 0), ((2, 1), 2)])
def test_progressive_decodes_like_baseline(script, hv, restart):
    """The same quantised coefficients written as a progressive sequence of
    scans decode to exactly the pixels of the baseline file."""
    img = _image(29, 45, seed=7 + script)
    q = np.arange(1, 65, dtype=np.int64) // 8 + 1  # small steps: many coefficients, deep refinement
    base = jpegio.read_jpeg(encode(img, hv=hv, q=q))[2]
    prog = jpegio.read_jpeg(encode(img, hv=hv, q=q, restart=restart, progressive=PROGRESSIVE[script]))[2]
    assert np.array_equal(base, prog)


def test_progressive_grey():
    img = _image(17, 26, seed=9)[..., 0]
    q = np.full(64, 1, np.int64)
    base = jpegio.read_jpeg(encode(img, q=q))[2]
    prog = jpegio.read_jpeg(encode(img, q=q, restart=1, progressive=PROGRESSIVE[1]))[2]
    assert np.array_equal(base, prog)


def test_rejects_what_the_cli_rejects():
    img = _image(8, 8, seed=1)
    data = bytearray(encode(img))
    i = data.index(b"\xff\xc0")
    data[i + 1] = 0xC9  # arithmetic coding
    with pytest.raises(jpegio.JpegError):
        jpegio.read_jpeg(bytes(data))
    with pytest.raises(jpegio.JpegError):
        jpegio.read_jpeg(b"not a jpeg")
    # four components (CMYK)
    cmyk = bytearray(encode(img))
    j = cmyk.index(b"\xff\xc0")
    seg_len = struct.unpack(">H", cmyk[j + 2:j + 4])[0]
    sof = cmyk[j + 4:j + 2 + seg_len]
    sof[5] = 4
    sof += bytes([4, 0x11, 0])
    cmyk[j:j + 2 + seg_len] = b"\xff\xc0" + struct.pack(">H", 2 + len(sof)) + bytes(sof)
    with pytest.raises(jpegio.JpegError):
        jpegio.read_jpeg(bytes(cmyk))


def test_read_image_picks_the_decoder_by_extension(tmp_path):
    from texpresso_gb300 import image, pngio
    img = _image(12, 20, seed=6)
    jp = tmp_path / "a.JPG"
    jp.write_bytes(encode(img))
    w, h, rgba = image.read_image(jp)
    assert (w, h) == (20, 12) and np.abs(rgba[..., :3].astype(int) - img).mean() < 3
    rgba4 = np.concatenate([img, np.full((12, 20, 1), 255, np.uint8)], -1)
    pn = tmp_path / "b.png"
    pngio.write_png(str(pn), 20, 12, rgba4)
    assert np.array_equal(image.read_image(pn)[2], rgba4)
    for bad in ("c.bmp", "noext"):
        with pytest.raises(ValueError):
            image.read_image(tmp_path / bad)


def test_progressive_long_end_of_band_runs():
    """A nearly flat image under coarse steps: most blocks end their bands at
    once, so the AC scans are mostly end-of-band runs across blocks."""
    img = np.full((64, 64, 3), 100, np.uint8)
    img[::7] = 140
    q = np.full(64, 40, np.int64)
    base = jpegio.read_jpeg(encode(img, q=q))[2]
    for script in PROGRESSIVE:
        assert np.array_equal(jpegio.read_jpeg(encode(img, q=q, progressive=script))[2], base)
