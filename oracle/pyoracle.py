"""Second CPU restatement of the reference block encoder (test infrastructure).

Independent of oracle/texpresso_oracle.c in structure: every ClusterFit
candidate of an ordering is evaluated at once with numpy float32 arrays
(each elementwise op rounds once, as the reference's scalar f32 ops do), the
winner is the first index holding the minimum of the errors strictly below
the running best, and RangeFit / alpha / packing use vectorised numpy.  Only
the running sums keep their sequential order (np.add.accumulate).  The test
suite checks this module and the C oracle against each other on thousands of
blocks, which guards each against slips in the other where the reference's
own known-answer tests (lib/src/test_data.rs) do not reach.

Reference: jansol/texpresso 2.0.2, lib/src/ (files cited per function).
"""
import math

import numpy as np

f32 = np.float32
F32_MAX = f32(np.finfo(np.float32).max)
EPS = f32(np.finfo(np.float32).eps)


def _roundf(x):
    """libm roundf (half away from zero), exact via double."""
    xd = float(x)
    return f32(math.copysign(math.floor(abs(xd) + 0.5), xd))


def _clamped(a, limit):
    """f32_to_i32_clamped (lib/src/math.rs:100-102)."""
    return int(np.fmin(np.fmax(_roundf(a), f32(0)), f32(limit)))


# --------------------------------------------------------------------------
# single-colour tables (lib/src/colourfit/single_lut.rs), libsquish generator

def _lut(bits, colours):
    err = np.full((256, 2), 255, np.int32)
    st = np.zeros((256, 2), np.int32)
    en = np.zeros((256, 2), np.int32)
    n = 1 << bits
    for v1 in range(n):
        a = (v1 << (8 - bits)) | (v1 >> (2 * bits - 8))
        for v2 in range(n):
            b = (v2 << (8 - bits)) | (v2 >> (2 * bits - 8))
            for k, t in enumerate((a, (a + b) // 2 if colours == 3 else (2 * a + b) // 3)):
                if err[t, k] != 0:
                    st[t, k], en[t, k], err[t, k] = v1, v2, 0
    changed = True
    while changed:
        changed = False
        for k in range(2):
            for t in range(256):
                for u in (t + 1, t - 1):
                    if 0 <= u < 256 and err[t, k] > err[u, k] + 1:
                        st[t, k], en[t, k], err[t, k] = st[u, k], en[u, k], err[u, k] + 1
                        changed = True
    return st, en, err


_LUTS = None


def luts():
    global _LUTS
    if _LUTS is None:
        _LUTS = [_lut(5, 3), _lut(6, 3), _lut(5, 4), _lut(6, 4)]
    return _LUTS


# --------------------------------------------------------------------------
# colour set (lib/src/colourset.rs:35-141)

def colour_set(px, mask, fmt, alpha_weighted):
    pts, wts, remap, transparent = [], [], [-1] * 16, False
    first_of = {}
    for i in range(16):
        if not (mask >> i) & 1:
            continue
        r, g, b, a = (int(c) for c in px[i])
        if fmt == 0 and a < 128:
            transparent = True
            continue
        w = f32(f32(a + 1) / f32(256)) if alpha_weighted else f32(1)
        key = (r, g, b)
        if key in first_of:
            idx = first_of[key]
            wts[idx] = f32(wts[idx] + w)
            remap[i] = idx
        else:
            first_of[key] = len(pts)
            remap[i] = len(pts)
            pts.append([f32(f32(r) / f32(255)), f32(f32(g) / f32(255)), f32(f32(b) / f32(255))])
            wts.append(w)
    wts = [f32(np.sqrt(w)) for w in wts]
    return np.array(pts, np.float32).reshape(-1, 3), np.array(wts, np.float32), remap, transparent


def _remap(remap, source):
    return [3 if r < 0 else int(source[r]) for r in remap]


# --------------------------------------------------------------------------
# math (lib/src/math.rs:44-97)

def principal(pts, wts):
    n = len(pts)
    total = f32(0)
    for w in wts:
        total = f32(total + w)
    c = np.zeros(3, np.float32)
    for i in range(n):
        c = (c + pts[i] * wts[i]).astype(np.float32)
    if total > EPS:
        c = (c / total).astype(np.float32)
    m = np.zeros(6, np.float32)
    for i in range(n):
        a = (pts[i] - c).astype(np.float32)
        b = (a * wts[i]).astype(np.float32)
        m = (m + np.array([a[0] * b[0], a[0] * b[1], a[0] * b[2], a[1] * b[1], a[1] * b[2], a[2] * b[2]],
                          np.float32)).astype(np.float32)
    rows = np.array([[m[0], m[1], m[2]], [m[1], m[3], m[4]], [m[2], m[4], m[5]]], np.float32)
    v = np.ones(3, np.float32)
    with np.errstate(all="ignore"):
        for _ in range(8):
            w = (rows[0] * v[0]).astype(np.float32)
            w = (rows[1] * v[1] + w).astype(np.float32)
            w = (rows[2] * v[2] + w).astype(np.float32)
            a = np.fmax(w[0], np.fmax(w[1], w[2]))
            v = (w * f32(f32(1) / a)).astype(np.float32)
    return v


def _dot(p, axis):
    with np.errstate(all="ignore"):
        return f32(f32(f32(p[0] * axis[0]) + f32(p[1] * axis[1])) + f32(p[2] * axis[2]))


# --------------------------------------------------------------------------
# packing (lib/src/colourblock.rs:28-94)

def _pack565(c):
    return (_clamped(f32(31) * c[0], 31) << 11) | (_clamped(f32(63) * c[1], 63) << 5) | _clamped(f32(31) * c[2], 31)


def _block(a, b, idx):
    out = bytearray(8)
    out[0:2] = a.to_bytes(2, "little")
    out[2:4] = b.to_bytes(2, "little")
    for i in range(4):
        out[4 + i] = (idx[4 * i] & 3) | ((idx[4 * i + 1] & 3) << 2) | ((idx[4 * i + 2] & 3) << 4) | ((idx[4 * i + 3] & 3) << 6)
    return bytes(out)


def write3(s, e, idx):
    a, b = _pack565(s), _pack565(e)
    if a > b:
        a, b = b, a
        idx = [1 if x == 0 else 0 if x == 1 else x for x in idx]
    return _block(a, b, idx)


def write4(s, e, idx):
    a, b = _pack565(s), _pack565(e)
    if a < b:
        a, b = b, a
        idx = [(x ^ 1) & 3 for x in idx]
    elif a == b:
        idx = [0] * 16
    return _block(a, b, idx)


# --------------------------------------------------------------------------
# fits

def single_fit(pts, remap, transparent, fmt):
    """lib/src/colourfit/single.rs:58-164"""
    col = [_clamped(pts[0][c] * f32(255), 255) for c in range(3)]
    best_err, best = 0xFFFFFFFF, bytes(8)
    passes = [(3, (0, 1, 0))] if fmt == 0 else []
    if fmt != 0 or not transparent:
        passes.append((4, (2, 3, 2)))
    for ncol, tabs in passes:
        err_i, sel = 0xFFFFFFFF, None
        for index in range(2):
            e = 0
            for c in range(3):
                e += int(luts()[tabs[c]][2][col[c], index]) ** 2
            if e < err_i:
                err_i, sel = e, index
        grid = (f32(31), f32(63), f32(31))
        s = [f32(f32(luts()[tabs[c]][0][col[c], sel]) / grid[c]) for c in range(3)]
        en = [f32(f32(luts()[tabs[c]][1][col[c], sel]) / grid[c]) for c in range(3)]
        if err_i < best_err:
            idx = _remap(remap, [2 * sel] * 16)
            best = write3(s, en, idx) if ncol == 3 else write4(s, en, idx)
            best_err = err_i
    return best


def _snap(x, grid, rcp):
    x = np.fmin(np.ones_like(x), np.fmax(np.zeros_like(x), x))
    return (np.trunc((grid * x + f32(0.5)).astype(np.float32)) * rcp).astype(np.float32)


GRID = np.array([31, 63, 31], np.float32)
GRIDRCP = np.array([f32(1) / f32(31), f32(1) / f32(63), f32(1) / f32(31)], np.float32)


def range_fit(pts, wts, remap, transparent, fmt, weights):
    """lib/src/colourfit/range.rs:44-192"""
    axis = principal(pts, wts)
    s = e = np.zeros(3, np.float32)
    if len(pts):
        s = e = pts[0]
        mn = mx = _dot(pts[0], axis)
        for p in pts[1:]:
            d = _dot(p, axis)
            if d < mn:
                s, mn = p, d
            elif d > mx:
                e, mx = p, d
    s, e = _snap(s, GRID, GRIDRCP), _snap(e, GRID, GRIDRCP)
    w = np.array(weights, np.float32)
    best_err, best = F32_MAX, bytes(8)
    passes = []
    if fmt == 0:
        passes.append((3, [s, e, (s * f32(0.5) + e * f32(0.5)).astype(np.float32)]))
    if fmt != 0 or not transparent:
        c23, c13 = f32(f32(2) / f32(3)), f32(f32(1) / f32(3))
        passes.append((4, [s, e, (s * c23 + e * c13).astype(np.float32), (s * c13 + e * c23).astype(np.float32)]))
    for ncol, codes in passes:
        closest, err = [], f32(0)
        for p in pts:
            dist, idx = F32_MAX, 0
            for j, c in enumerate(codes):
                d = (w * (p - c).astype(np.float32)).astype(np.float32)
                dd = f32(f32(f32(d[0] * d[0]) + f32(d[1] * d[1])) + f32(d[2] * d[2]))
                if dd < dist:
                    dist, idx = dd, j
            closest.append(idx)
            err = f32(err + dist)
        if err < best_err:
            idx = _remap(remap, closest)
            best = write3(s, e, idx) if ncol == 3 else write4(s, e, idx)
            best_err = err
    return best


def _order(pts, axis):
    """Stable sort of 16 entries, non-finite dots last (cluster.rs:84-100)."""
    keys = []
    for i in range(16):
        d = _dot(pts[i], axis) if i < len(pts) else F32_MAX
        keys.append((1, 0.0) if not np.isfinite(d) else (0, float(d)))
    ix = sorted(range(16), key=lambda t: keys[t])       # Python's sort is stable
    return [ix_ if ix_ < len(pts) else 0 for ix_ in ix]


def _candidates(n, ncol):
    if ncol == 4:
        return [(i, j, k) for i in range(n) for j in range(i, n + 1) for k in range(max(j, 1), n + 1)]
    return [(i, j, 0) for i in range(n) for j in range(max(i, 1), n + 1)]


def _fit_all(P0, P1, P2, xs, w, ncol):
    """Evaluate every candidate (arrays of shape (m, 4)) at once."""
    with np.errstate(all="ignore"):
        if ncol == 4:
            c13 = np.array([f32(1) / f32(3)] * 3 + [f32(1) / f32(9)], np.float32)
            c23 = np.array([f32(2) / f32(3)] * 3 + [f32(4) / f32(9)], np.float32)
            P3 = (((xs - P2).astype(np.float32) - P1).astype(np.float32) - P0).astype(np.float32)
            ax = ((P2 * c13).astype(np.float32) + ((P1 * c23).astype(np.float32) + P0).astype(np.float32)).astype(np.float32)
            bx = ((P1 * c13).astype(np.float32) + ((P2 * c23).astype(np.float32) + P3).astype(np.float32)).astype(np.float32)
            ab = (f32(f32(2) / f32(9)) * (P1[:, 3] + P2[:, 3]).astype(np.float32)).astype(np.float32)
        else:
            hh = np.array([0.5, 0.5, 0.5, 0.25], np.float32)
            P2 = ((xs - P1).astype(np.float32) - P0).astype(np.float32)
            t = (P1 * hh).astype(np.float32)
            ax = (t + P0).astype(np.float32)
            bx = (t + P2).astype(np.float32)
            ab = t[:, 3]
        a2, b2 = ax[:, 3], bx[:, 3]
        factor = (f32(1) / ((a2 * b2).astype(np.float32) - (ab * ab).astype(np.float32)).astype(np.float32)).astype(np.float32)
        A = (((ax[:, :3] * b2[:, None]).astype(np.float32) - (bx[:, :3] * ab[:, None]).astype(np.float32)).astype(np.float32)
             * factor[:, None]).astype(np.float32)
        B = (((bx[:, :3] * a2[:, None]).astype(np.float32) - (ax[:, :3] * ab[:, None]).astype(np.float32)).astype(np.float32)
             * factor[:, None]).astype(np.float32)
        A, B = _snap(A, GRID, GRIDRCP), _snap(B, GRID, GRIDRCP)
        e1 = (((A * A).astype(np.float32) * a2[:, None]).astype(np.float32)
              + ((B * B).astype(np.float32) * b2[:, None]).astype(np.float32)).astype(np.float32)
        e2 = ((((A * B).astype(np.float32) * ab[:, None]).astype(np.float32))
              - (A * ax[:, :3]).astype(np.float32)).astype(np.float32)
        e3 = (e2 - (B * bx[:, :3]).astype(np.float32)).astype(np.float32)
        e4 = ((f32(2) * e3).astype(np.float32) + e1).astype(np.float32)
        e5 = (e4 * w).astype(np.float32)
        err = ((e5[:, 0] + e5[:, 1]).astype(np.float32) + e5[:, 2]).astype(np.float32)
    return err, A, B


def cluster_fit(pts, wts, remap, transparent, fmt, weights, iterate):
    """lib/src/colourfit/cluster.rs:33-417 with lib/src/colourfit.rs:44-60"""
    n = len(pts)
    w = np.array(weights, np.float32)
    principal_axis = principal(pts, wts)
    best_err, best = F32_MAX, bytes(8)
    passes = [3] if fmt == 0 else []
    if fmt != 0 or not transparent:
        passes.append(4)
    for ncol in passes:
        run = best_err
        ba = bb = np.zeros(3, np.float32)
        best_it, best_c, orders = 0, None, []
        axis = principal_axis
        cands = _candidates(n, ncol)
        for it in range(8 if iterate else 1):
            order = _order(pts, axis)
            if order in orders:
                orders.append(order)
                break
            orders.append(order)
            pw = np.zeros((16, 4), np.float32)
            for m in range(n):
                j = order[m]
                pw[m] = (np.array([pts[j][0], pts[j][1], pts[j][2], 1], np.float32) * wts[j]).astype(np.float32)
            S = np.zeros((17, 17, 4), np.float32)
            for a in range(n):
                S[a, a + 1:n + 1] = np.add.accumulate(pw[a:n], axis=0, dtype=np.float32)
            xs = S[0, n]
            I = np.array([c[0] for c in cands])
            J = np.array([c[1] for c in cands])
            K = np.array([c[2] for c in cands])
            P0, P1 = S[0, I], S[I, J]
            P2 = S[J, K] if ncol == 4 else None
            err, A, B = _fit_all(P0, P1, P2, xs, w, ncol)
            below = err < run            # NaN never qualifies; -inf does
            if below.any():
                ok = np.where(below, err, np.inf)
                t = int(np.argmin(ok))   # first position of the minimum
                run, ba, bb, best_it, best_c = ok[t], A[t], B[t], it, cands[t]
            if best_it != it:
                break
            axis = (bb - ba).astype(np.float32)
        if run < best_err:
            i, j, k = best_c
            order = orders[best_it]
            un = [0] * 16
            for m in range(i, j):
                un[order[m]] = 2
            for m in range(j, n):
                un[order[m]] = 1 if ncol == 3 else 3
            if ncol == 4:
                for m in range(k, n):
                    un[order[m]] = 1
            idx = _remap(remap, un)
            best = write3(ba, bb, idx) if ncol == 3 else write4(ba, bb, idx)
            best_err = run
    return best


# --------------------------------------------------------------------------
# alpha (lib/src/alpha.rs:27-256)

def bc2_alpha(px, mask):
    out = bytearray(8)
    for i in range(8):
        q = [0 if not (mask >> p) & 1 else _clamped(f32(int(px[p][3])) * f32(f32(15) / f32(255)), 15)
             for p in (2 * i, 2 * i + 1)]
        out[i] = q[0] | (q[1] << 4)
    return bytes(out)


def codes7(min5, max5, min7, max7):
    """The 7-value codebook; its first two entries are the 5-mode endpoints
    (lib/src/alpha.rs:237-242)."""
    return np.array([min5, max5] + [((7 - i) * min7 + i * max7) // 7 for i in range(1, 7)])


def bc3_alpha(px, ch, mask):
    vals = np.array([int(px[i][ch]) for i in range(16)])
    valid = np.array([(mask >> i) & 1 for i in range(16)], bool)
    v = vals[valid]
    min7, max7 = (int(v.min()), int(v.max())) if v.size else (255, 0)
    nz, n255 = v[v != 0], v[v != 255]
    min5 = int(nz.min()) if nz.size else 255
    max5 = int(n255.max()) if n255.size else 0
    min5 = min(min5, max5)
    min7 = min(min7, max7)

    def fix(lo, hi, steps):
        if hi - lo < steps:
            hi = min(lo + steps, 255)
        if hi - lo < steps:
            lo = max(hi - steps, 0)
        return lo, hi
    min5, max5 = fix(min5, max5, 5)
    min7, max7 = fix(min7, max7, 7)
    c5 = np.array([min5, max5] + [((5 - i) * min5 + i * max5) // 5 for i in range(1, 5)] + [0, 255])
    c7 = codes7(min5, max5, min7, max7)

    def fit(codes):
        d = (vals[:, None] - codes[None, :]) ** 2
        idx = np.argmin(d, axis=1)                       # first minimum
        least = d[np.arange(16), idx]
        idx = np.where(valid, idx, 0)
        return int(np.where(valid, least, 0).sum()), idx

    e5, i5 = fit(c5)
    e7, i7 = fit(c7)
    if e5 <= e7:
        a0, a1, idx = min5, max5, i5
        if a0 > a1:
            a0, a1 = a1, a0
            idx = np.array([1 if x == 0 else 0 if x == 1 else (7 - x if 2 <= x <= 5 else x) for x in idx])
    else:
        a0, a1, idx = min7, max7, i7
        if a0 < a1:
            a0, a1 = a1, a0
            idx = np.array([1 if x == 0 else 0 if x == 1 else 9 - x for x in idx])
    bits = 0
    for p in range(16):
        bits |= int(idx[p]) << (3 * p)
    return bytes([a0, a1]) + bits.to_bytes(6, "little")


def compress_block_masked(fmt, rgba64, mask, algorithm, weights, alpha_weighted):
    """lib/src/lib.rs:188-234"""
    px = np.asarray(rgba64, np.uint8).reshape(16, 4)
    out = b""
    if fmt == 1:
        out = bc2_alpha(px, mask)
    elif fmt == 2:
        out = bc3_alpha(px, 3, mask)
    elif fmt == 3:
        return bc3_alpha(px, 0, mask)
    elif fmt == 4:
        return bc3_alpha(px, 0, mask) + bc3_alpha(px, 1, mask)
    pts, wts, remap, transparent = colour_set(px, mask, fmt, alpha_weighted)
    if len(pts) == 1:
        col = single_fit(pts, remap, transparent, fmt)
    elif algorithm == 0 or len(pts) == 0:
        col = range_fit(pts, wts, remap, transparent, fmt, weights)
    else:
        col = cluster_fit(pts, wts, remap, transparent, fmt, weights, algorithm == 2)
    return out + col
