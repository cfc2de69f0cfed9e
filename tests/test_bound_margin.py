"""The ClusterFit pruning bounds (cand_bound / lb_terms, and unit_bound /
unit_terms for 16 colours of weight 1, in texpresso_gb300/csrc/tx_colour.cuh),
restated in numpy, never exceeds the
reference's error (the numpy oracle's f32 evaluation) on any candidate of
natural, palette and 5:6:5-grid blocks under several weight sets, with and
without alpha weighting.  FMA steps are emulated in double and rounded once,
as the device does.  The margin's slack is reported: every candidate must
keep E - bound >= 0, and the unmargined bound may dip below E only by part of
the margin."""
import numpy as np

from oracle import pyoracle as po
from texpresso_gb300 import workloads

f32 = np.float32


def fma(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64)).astype(np.float32)


def bounds(P0, P1, P2, xs, w, nc):
    """(bound with margin, bound without, margin) per candidate, as the kernel computes them."""
    if nc == 4:
        ax = fma(P2[:, :3], f32(1 / 3), fma(P1[:, :3], f32(2 / 3), P0[:, :3]))
        p3w = (((xs[3] - P0[:, 3]).astype(f32) - P1[:, 3]).astype(f32) - P2[:, 3]).astype(f32)
        al = fma(P2[:, 3], f32(1 / 9), fma(P1[:, 3], f32(4 / 9), P0[:, 3]))
        be = fma(P1[:, 3], f32(1 / 9), fma(P2[:, 3], f32(4 / 9), p3w))
        g2 = (f32(4 / 9) * (P1[:, 3] + P2[:, 3]).astype(f32)).astype(f32)
    else:
        ax = fma(P1[:, :3], f32(0.5), P0[:, :3])
        p2w = ((xs[3] - P0[:, 3]).astype(f32) - P1[:, 3]).astype(f32)
        al = fma(P1[:, 3], f32(0.25), P0[:, 3])
        be = fma(P1[:, 3], f32(0.25), p2w)
        g2 = (f32(0.5) * P1[:, 3]).astype(f32)
    g = (f32(0.5) * g2).astype(f32)
    det = (al.astype(np.float64) * be - g.astype(np.float64) ** 2).astype(f32)
    # the quadratic in ax alone (bx = X - ax): A = alpha + beta + 2 gamma, B2 = -2 (alpha + gamma)
    A = (al.astype(np.float64) + be + g2).astype(f32)
    B2 = (-(2.0 * al.astype(np.float64) + g2)).astype(f32)
    with np.errstate(all="ignore"):
        f = np.where(det > 0, (f32(1) / det).astype(f32), np.nan).astype(f32)
        wx = (w * ax).astype(f32)
        s1 = (wx[:, 0] * ax[:, 0]).astype(f32)
        s1 = fma(wx[:, 1], ax[:, 1], s1)
        s1 = fma(wx[:, 2], ax[:, 2], s1)
        wX = (w * xs[:3]).astype(f32)
        s2 = (wX[0] * ax[:, 0]).astype(f32)
        s2 = fma(wX[1], ax[:, 1], s2)
        s2 = fma(wX[2], ax[:, 2], s2)
        Z = f32(0)
        for c in range(3):
            Z = fma(w[c], (xs[c] * xs[c]).astype(f32), Z)
        kb = f32(2.0 ** -17) * xs[3] * Z
        eps1 = f32(2.0 ** -17) * xs[3] * f32(w.sum())
        acc = fma(A, s1, fma(B2, s2, fma(al, Z, kb)))
        lbm = fma(-f, acc, -eps1)
        acc0 = fma(A, s1, fma(B2, s2, (al * Z).astype(f32)))
        lb0 = (-f * acc0).astype(f32)
        margin = (f * kb + eps1).astype(f32)
        # one-cluster candidates get the flat bound -(1 + 2^-10) Z / W - eps1
        cnt = [P0[:, 3], P1[:, 3], P2[:, 3]] if nc == 4 else [P0[:, 3], P1[:, 3]]
        one = sum((c == xs[3]).astype(int) for c in cnt) == 1
        rw = (f32(1) / xs[3]).astype(f32)
        lbm = np.where(one, fma((-(f32(1) + f32(2.0 ** -10)) * Z).astype(f32), rw, -eps1), lbm)
        lb0 = np.where(one, (-Z * rw).astype(f32), lb0)
        margin = np.where(one, (f32(2.0 ** -10) * Z * rw + eps1).astype(f32), margin)
    return lbm, lb0, margin


def wterms(P0w, P1w, P2w, xsw, nc):
    """The reference's f32 alpha2, beta2, alphabeta (wterms4 / wterms3)."""
    if nc == 4:
        p3w = (((xsw - P2w).astype(f32) - P1w).astype(f32) - P0w).astype(f32)
        al = ((P2w * f32(1 / 9)).astype(f32) + ((P1w * f32(4 / 9)).astype(f32) + P0w).astype(f32)).astype(f32)
        be = ((P1w * f32(1 / 9)).astype(f32) + ((P2w * f32(4 / 9)).astype(f32) + p3w).astype(f32)).astype(f32)
        ab = (f32(2 / 9) * (P1w + P2w).astype(f32)).astype(f32)
    else:
        p2w = ((xsw - P1w).astype(f32) - P0w).astype(f32)
        al = fma(P1w, f32(0.25), P0w)
        be = fma(P1w, f32(0.25), p2w)
        ab = (P1w * f32(0.25)).astype(f32)
    return al, be, ab


def unit_bounds(P0, P1, P2, xs, w, nc):
    """unit_bound with the unit_terms table, as the kernel computes it for a
    16-colour set of weight-1 points."""
    al, be, ga = (v.astype(np.float64) for v in wterms(P0[:, 3], P1[:, 3], P2[:, 3], xs[3], nc))
    det = al * be - ga * ga
    A = al + be + 2 * ga
    # every point in one cluster: the flat bound -(1 + 2^-10) Z / 16
    cnt = [P0[:, 3], P1[:, 3], P2[:, 3]] if nc == 4 else [P0[:, 3], P1[:, 3]]
    one = sum((c == 16).astype(int) for c in cnt) + (xs[3] - sum(cnt) == 16).astype(int) == 1
    flat = ~(det > 0) & one
    with np.errstate(all="ignore"):
        F1 = np.where(det > 0, -A / det, np.where(flat, 0, np.nan)).astype(f32)
        r = np.where(det > 0, 2 * (al + ga) / A, 0).astype(f32)
        C = np.where(det > 0, -(al + 2.0 ** -13) / det, np.where(flat, -(1 + 2.0 ** -10) / 16, np.nan)).astype(f32)
        C0 = np.where(det > 0, -al / det, np.where(flat, -1 / 16, np.nan)).astype(f32)
        f = np.where(det > 0, 1 / det, np.where(flat, 2.0 ** -10 / 16 / 2.0 ** -13, np.nan)).astype(f32)
        if nc == 4:
            ax = fma(P2[:, :3], f32(1 / 3), fma(P1[:, :3], f32(2 / 3), P0[:, :3]))
        else:
            ax = fma(P1[:, :3], f32(0.5), P0[:, :3])
        d = fma(-r[:, None], xs[None, :3], ax)
        cwax = (w * ax).astype(f32)
        sm = (cwax[:, 0] * d[:, 0]).astype(f32)
        sm = fma(cwax[:, 1], d[:, 1], sm)
        sm = fma(cwax[:, 2], d[:, 2], sm)
        Z = f32(0)
        for c in range(3):
            Z = fma(w[c], (xs[c] * xs[c]).astype(f32), Z)
        eps1 = f32(2.0 ** -17) * xs[3] * f32(w.sum())
        lbm = fma(F1, sm, fma(C, Z, -eps1))
        lb0 = fma(F1, sm, (C0 * Z).astype(f32))
        margin = (f * (f32(2.0 ** -17) * xs[3] * Z) + eps1).astype(f32)
    return lbm, lb0, margin


def blocks():
    img = workloads.ramp_texture(64, 64, seed=9, alpha="ramp")
    nat = workloads.image_to_blocks(img)[0]
    return np.concatenate([nat, workloads.grid_blocks(200, seed=10), workloads.random_blocks(150, seed=11)])


def test_bound_never_exceeds_reference_error():
    total, worst, n_unit = 0, np.inf, 0
    for bi, blk in enumerate(blocks()):
        w = [np.array([0.2126, 0.7152, 0.0722], f32), np.array([1, 1, 1], f32),
             np.array([0.0, 1.0, 0.001], f32)][bi % 3]
        pts, wts, _, _ = po.colour_set(blk.reshape(16, 4), 0xFFFF, 2, bi % 4 == 3)
        n = len(pts)
        if n < 2:
            continue
        order = po._order(pts, po.principal(pts, wts))
        pw = np.zeros((16, 4), f32)
        for m in range(n):
            j = order[m]
            pw[m] = (np.array([pts[j][0], pts[j][1], pts[j][2], 1], f32) * wts[j]).astype(f32)
        S = np.zeros((17, 17, 4), f32)
        for a in range(n):
            S[a, a + 1:n + 1] = np.add.accumulate(pw[a:n], axis=0, dtype=f32)
        xs = S[0, n]
        for nc in (4, 3):
            cands = po._candidates(n, nc)
            I = np.array([c[0] for c in cands]); J = np.array([c[1] for c in cands])
            K = np.array([c[2] for c in cands])
            P0, P1 = S[0, I], S[I, J]
            P2 = S[J, K] if nc == 4 else np.zeros_like(P0)
            err, _, _ = po._fit_all(P0, P1, P2 if nc == 4 else None, xs, w, nc)
            forms = [bounds(P0, P1, P2, xs, w, nc)]
            if n == 16 and np.all(wts == 1):
                forms.append(unit_bounds(P0, P1, P2, xs, w, nc))
                n_unit += 1
            for lbm, lb0, margin in forms:
                ok = np.isfinite(lbm) & ~np.isnan(err)  # a NaN error never wins
                assert np.all(err[ok] >= lbm[ok]), (bi, nc)
                total += int(ok.sum())
                if ok.any():
                    worst = min(worst, float(np.min((err[ok] - lb0[ok]) / margin[ok])))
    assert total > 100000
    assert n_unit > 100
    # the unmargined bound may fall below the error by rounding, never by more
    # than a small part of the margin
    assert worst > -0.25, worst
