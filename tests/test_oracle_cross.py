"""The C oracle against the second, vectorised restatement (oracle/pyoracle.py)
on seeded adversarial blocks: every format and algorithm, partial masks,
three weight sets, alpha weighting on and off.  The two restatements share no
code, so agreement here covers the ClusterFit orderings, the 3- and 4-colour
candidate sweeps, the iteration stop rule and the alpha codebook tie rules at
many more points than the reference's eight known-answer blocks."""
import numpy as np
import pytest

from oracle import pyoracle
from texpresso_gb300 import workloads

WEIGHTS = [(0.2126, 0.7152, 0.0722), (1.0, 1.0, 1.0), (0.5, 0.0, 2.0)]


def _blocks(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for t in range(n):
        kind = t % 6
        if kind == 0:            # uniform noise
            b = rng.integers(0, 256, 64)
        elif kind == 1:          # few levels: many duplicate colours and ties
            b = rng.integers(0, 4, 64) * 85
        elif kind == 2:          # three-colour palette
            b = rng.integers(0, 256, (3, 4))[rng.integers(0, 3, 16)].reshape(64)
        elif kind == 3:          # near-flat block
            b = np.clip(rng.integers(0, 256, 4) + rng.integers(-3, 4, (16, 4)), 0, 255).reshape(64)
        elif kind == 4:          # alpha around the BC1 threshold and the extremes
            b = rng.integers(0, 256, 64)
            b[3::4] = rng.choice([0, 127, 128, 255], 16)
        else:                    # two-colour gradient
            lo, hi = rng.integers(0, 256, 4), rng.integers(0, 256, 4)
            t16 = np.linspace(0, 1, 16)[:, None]
            b = np.round(lo + (hi - lo) * t16).astype(np.int64).reshape(64)
        out.append(b.astype(np.uint8))
    return out


def _cases(n, seed):
    rng = np.random.default_rng(seed + 1)
    for i, b in enumerate(_blocks(n, seed)):
        mask = 0xFFFF if i % 3 else int(rng.integers(0, 1 << 16))
        for fmt in range(5):
            for alg in range(3) if fmt < 3 else (0,):
                yield b, mask, fmt, alg, WEIGHTS[i % 3], bool(i % 2)


def test_restatements_agree(oracle):
    bad = []
    for b, mask, fmt, alg, w, aw in _cases(600, 7):
        ref = bytes(oracle.compress_block_masked(fmt, b, mask, oracle.make_params(alg, w, aw)))
        got = pyoracle.compress_block_masked(fmt, b, mask, alg, w, aw)
        if ref != got:
            bad.append((fmt, alg, hex(mask), ref.hex(), got.hex()))
    assert not bad, bad[:5]


def test_restatement_matches_kat(kat):
    formats = {"BC1": 0, "BC2": 1, "BC3": 2, "BC4": 3, "BC5": 4}
    algos = {"RangeFit": 0, "ClusterFit": 1, "IterativeClusterFit": 2}
    w = kat["compression_params"]["weights"]
    for name, d in kat["datasets"].items():
        fmt = formats[d["format"]]
        for alg in kat["compression_params"]["algorithms"]:
            got = pyoracle.compress_block_masked(fmt, np.array(d["decoded"], np.uint8), 0xFFFF,
                                                 algos[alg], w, False)
            assert list(got) == d["encoded"], (name, alg)


EXTREME_WEIGHTS = [(1.0, 0.0, 0.0), (0.0, 0.0, 0.0), (1e-40, 1.0, 1e-3), (1e6, 1e6, 1e6), (3e38, 1.0, 1.0),
                   (-1.0, 1.0, 1.0), (float("inf"), 1.0, 1.0), (float("nan"), 1.0, 1.0)]


def test_restatements_agree_on_grid_blocks_and_extreme_weights(oracle):
    """Colours on the 5:6:5 grid and weights that are zero, subnormal, huge,
    negative or non-finite (errors of -inf or NaN take the reference's
    "strictly smaller" rule)."""
    blocks = workloads.grid_blocks(60, seed=3)
    bad = []
    with np.errstate(all="ignore"):
        for w in EXTREME_WEIGHTS:
            for alg in (0, 1, 2):
                for fmt in (0, 2):
                    for i, b in enumerate(blocks):
                        p = oracle.make_params(alg, w, bool(i % 2))
                        ref = bytes(oracle.compress_block_masked(fmt, b, 0xFFFF, p))
                        got = pyoracle.compress_block_masked(fmt, b, 0xFFFF, alg, w, bool(i % 2))
                        if ref != got:
                            bad.append((w, alg, fmt, i))
    assert not bad, bad[:5]


def test_cross_check_catches_a_planted_slip(oracle, monkeypatch):
    """A slip planted in the numpy restatement (the 7-value codebook seeded
    from its own endpoints instead of the 5-mode ones) must show up."""
    monkeypatch.setattr(pyoracle, "codes7", lambda min5, max5, min7, max7: np.array(
        [min7, max7] + [((7 - i) * min7 + i * max7) // 7 for i in range(1, 7)]))
    diffs = 0
    for b, mask, fmt, alg, w, aw in _cases(300, 11):
        if fmt != 3:
            continue
        ref = bytes(oracle.compress_block_masked(fmt, b, mask, oracle.make_params(alg, w, aw)))
        diffs += ref != pyoracle.compress_block_masked(fmt, b, mask, alg, w, aw)
    assert diffs > 0
