"""GPU parity: the CUDA kernels (through the C ABI) against the CPU oracle on
the reference's known-answer blocks, seeded synthetic textures of every
benchmark configuration, adversarial blocks, every mask of selected blocks,
odd image sizes and the decoders.

The bar (lib/src/lib.rs:188-335 as restated by the oracle): packed output is
bit-identical for SingleColourFit, RangeFit and the alpha paths; ClusterFit is
bit-identical, or a differing block decodes to a squared error within 1e-6
relative of the oracle's (a tie).  The identical fraction is printed.
"""
import numpy as np
import pytest

from texpresso_gb300 import workloads

pytestmark = pytest.mark.gpu

PERCEPTUAL = (0.2126, 0.7152, 0.0722)
UNIFORM = (1.0, 1.0, 1.0)
FMT_NAMES = ["BC1", "BC2", "BC3", "BC4", "BC5"]


def tx_params(tx, alg, weights=PERCEPTUAL, aw=False):
    return tx.Params(algorithm=tx.Algorithm(alg), weights=weights, weigh_colour_by_alpha=aw)


def dev_compress(tx, torch, fmt, img, params, channels=None, out_len=None):
    h, w = img.shape[:2]
    ch = channels or img.shape[2]
    t = torch.from_numpy(np.ascontiguousarray(img)).cuda()
    fmt = tx.Format(fmt)
    n = out_len or fmt.compressed_size(w, h)
    out = torch.zeros(n, dtype=torch.uint8, device="cuda")
    tx.compress_device(fmt, t.data_ptr(), w * ch, ch, w, h, params, out.data_ptr(), n,
                       torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def dev_compress_blocks(tx, torch, fmt, blocks, masks, params):
    b = torch.from_numpy(np.ascontiguousarray(blocks)).cuda()
    m = torch.from_numpy(np.ascontiguousarray(masks).view(np.int32)).cuda() if masks is not None else None
    fmt = tx.Format(fmt)
    out = torch.zeros(blocks.shape[0] * fmt.block_size(), dtype=torch.uint8, device="cuda")
    tx.compress_blocks_device(fmt, b.data_ptr(), m.data_ptr() if m is not None else 0, blocks.shape[0], params,
                              out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(blocks.shape[0], -1)


def block_error(oracle, fmt, enc, src, mask, weights):
    """Sum over valid, non-transparent pixels of sum_c w_c (dec - src)^2 (cluster.rs:219)."""
    dec = oracle.decompress_block(fmt, enc).reshape(16, 4).astype(np.float64)
    s = src.reshape(16, 4).astype(np.float64)
    e = 0.0
    for p in range(16):
        if not (mask >> p) & 1:
            continue
        if fmt == 0 and src.reshape(16, 4)[p, 3] < 128:
            continue
        e += sum(weights[c] * (dec[p, c] - s[p, c]) ** 2 for c in range(3))
    return e


def check_blocks(oracle, fmt, got, ref, blocks, masks, weights, cluster, label):
    got = got.reshape(ref.shape)
    diff = np.flatnonzero(np.any(got != ref, axis=1))
    ident = 1.0 - diff.size / max(1, ref.shape[0])
    print("%s: %d blocks, identical fraction %.6f" % (label, ref.shape[0], ident))
    if diff.size == 0:
        return
    assert cluster, "%s: %d blocks differ on a bit-exact path (first %d)" % (label, diff.size, diff[0])
    bs = ref.shape[1]
    for b in diff[:2000]:
        m = int(masks[b]) if masks is not None else 0xFFFF
        col = slice(0, 8) if fmt == 0 else slice(8, 16)
        assert np.array_equal(got[b, :8], ref[b, :8]) or fmt == 0, "%s: alpha differs in block %d" % (label, b)
        eg = block_error(oracle, fmt, got[b, :bs], blocks[b], m, weights)
        er = block_error(oracle, fmt, ref[b, :bs], blocks[b], m, weights)
        assert abs(eg - er) <= 1e-6 * max(er, 1e-12), "%s: block %d not a tie (%r vs %r)" % (label, b, eg, er)
        del col


# ---------------------------------------------------------------------------
# known answers (lib/src/lib.rs:395-504)

@pytest.mark.parametrize("name", ["BC1_GRAY", "BC1_COLOUR", "BC2_GRAY", "BC2_COLOUR", "BC3_GRAY",
                                  "BC3_COLOUR", "BC4_GRAY", "BC5_GRAY"])
def test_kat_compress(tx, cuda, kat, name):
    d = kat["datasets"][name]
    fmt = tx.Format(FMT_NAMES.index(d["format"]))
    for alg in kat["compression_params"]["algorithms"]:
        p = tx.Params(algorithm=tx.Algorithm[alg], weights=UNIFORM, weigh_colour_by_alpha=False)
        out = bytearray(fmt.block_size())
        fmt.compress(bytes(d["decoded"]), 4, 4, p, out)
        assert list(out) == d["encoded"], (name, alg)
        blk = bytearray(fmt.block_size())
        fmt.compress_block_masked(bytes(d["decoded"]), 0xFFFF, p, blk)
        assert list(blk) == d["encoded"], (name, alg, "masked")


@pytest.mark.parametrize("name", ["BC1_GRAY", "BC1_COLOUR", "BC2_GRAY", "BC2_COLOUR", "BC3_GRAY",
                                  "BC3_COLOUR", "BC4_GRAY", "BC5_GRAY"])
def test_kat_decompress(tx, cuda, kat, name):
    d = kat["datasets"][name]
    fmt = tx.Format(FMT_NAMES.index(d["format"]))
    out = bytearray(64)
    fmt.decompress(bytes(d["encoded"]), 4, 4, out)
    assert list(out) == d["decoded"]
    assert list(fmt.decompress_block(bytes(d["encoded"]))) == d["decoded"]


def test_kat_odd_height_decode(tx, cuda, kat):
    c = kat["odd_height_decode"]
    out = bytearray(c["width"] * c["height"] * 4)
    tx.Format.Bc1.decompress(bytes(c["encoded"]), c["width"], c["height"], out)
    assert np.frombuffer(bytes(out), np.uint8).reshape(-1, 4).tolist() == [c["pixel"]] * (c["width"] * c["height"])


# ---------------------------------------------------------------------------
# synthetic benchmark textures

def compare_image(tx, cuda, oracle, fmt, img, alg, weights=PERCEPTUAL, aw=False, label="", host=False,
                  strict=False):
    h, w = img.shape[:2]
    p = tx_params(tx, alg, weights, aw)
    if host:
        got = np.zeros(tx.Format(fmt).compressed_size(w, h), np.uint8)
        tx.Format(fmt).compress(img, w, h, p, got)
    else:
        got = dev_compress(tx, cuda, fmt, img, p)
    ref = oracle.compress(fmt, img, w, h, oracle.make_params(alg, weights, aw))
    if strict:
        bs = tx.Format(fmt).block_size()
        ndiff = int(np.any(got.reshape(-1, bs) != ref.reshape(-1, bs), axis=1).sum())
        assert ndiff == 0, "%s alg%d %dx%d aw%d: %d blocks differ (bit-identical required)" % (
            FMT_NAMES[fmt], alg, w, h, aw, ndiff)
        return
    blocks, masks = workloads.image_to_blocks(img)
    bs = tx.Format(fmt).block_size()
    check_blocks(oracle, fmt, got.reshape(-1, bs), ref.reshape(-1, bs), blocks, masks, weights, alg != 0,
                 label or "%s alg%d %dx%d aw%d" % (FMT_NAMES[fmt], alg, w, h, aw))


def test_c0_bc1_clusterfit_256(tx, cuda, oracle):
    img = workloads.ramp_texture(256, 256, seed=0)
    p = tx_params(tx, 1)
    got = dev_compress(tx, cuda, 0, img, p)
    ref = oracle.compress(0, img, 256, 256, oracle.make_params(1))
    assert np.array_equal(got, ref), "C0 BC1 ClusterFit: %d of 4096 blocks differ" % int(
        np.any(got.reshape(-1, 8) != ref.reshape(-1, 8), axis=1).sum())


@pytest.mark.parametrize("alg", [0, 1])
@pytest.mark.parametrize("aw", [False, True])
def test_c1_bc3_2048(tx, cuda, oracle, alg, aw):
    # bit-identical for RangeFit and ClusterFit alike (no tie allowance)
    img = workloads.ramp_texture(2048, 2048, seed=1, alpha="ramp")
    compare_image(tx, cuda, oracle, 2, img, alg, aw=aw, strict=True)


def test_c1_bc3_host_api_matches_device_api(tx, cuda, oracle):
    img = workloads.ramp_texture(1000, 600, seed=11, alpha="ramp")
    compare_image(tx, cuda, oracle, 2, img, 1, host=True, label="BC3 host API 1000x600")


@pytest.mark.parametrize("fmt", [0, 1, 2])
@pytest.mark.parametrize("alg", [0, 1, 2])
def test_formats_algorithms(tx, cuda, oracle, fmt, alg):
    img = workloads.ramp_texture(192, 160, seed=10 + fmt + 3 * alg, alpha="ramp" if fmt else "opaque")
    if fmt == 0:
        img[::7, ::5, 3] = 0  # some transparent pixels for BC1
    for weights in (PERCEPTUAL, UNIFORM):
        for aw in (False, True):
            compare_image(tx, cuda, oracle, fmt, img, alg, weights, aw)


def test_c2_bc4_bc5_4096(tx, cuda, oracle):
    r = workloads.value_noise(4096, 4096, channels=2, seed=3)
    rgba = workloads.expand_to_rgba(r)
    p = tx.Params()
    for fmt, ch in ((3, 1), (4, 2)):
        ref = oracle.compress(fmt, rgba, 4096, 4096, oracle.make_params())
        got = dev_compress(tx, cuda, fmt, rgba, p)
        assert np.array_equal(got, ref), "%s RGBA input differs" % FMT_NAMES[fmt]
        native = np.ascontiguousarray(r[..., :ch])
        got_n = dev_compress(tx, cuda, fmt, native, p, channels=ch)
        assert np.array_equal(got_n, ref), "%s native %d-channel input differs" % (FMT_NAMES[fmt], ch)
        # both codebooks must have been exercised
        blocks, masks = workloads.image_to_blocks(rgba[:256, :256])
        _, st = oracle.compress_blocks(fmt, blocks, masks, oracle.make_params(), with_stats=True)
        modes = set(st["alpha_mode"][:, 0].tolist())
        assert {5, 7} <= modes, modes


# ---------------------------------------------------------------------------
# adversarial blocks, masks, sizes

@pytest.mark.parametrize("fmt", [0, 1, 2, 3, 4])
def test_adversarial_blocks(tx, cuda, oracle, fmt):
    n = 6000
    blocks = workloads.random_blocks(n, seed=100 + fmt)
    rng = np.random.default_rng(7 + fmt)
    masks = np.where(rng.uniform(size=n) < 0.3, rng.integers(0, 1 << 16, size=n), 0xFFFF).astype(np.uint32)
    algs = [0, 1, 2] if fmt < 3 else [1]
    for alg in algs:
        for weights, aw in ((PERCEPTUAL, False), (UNIFORM, True), ((0.5, 0.3, 0.9), False)):
            p = tx_params(tx, alg, weights, aw)
            got = dev_compress_blocks(tx, cuda, fmt, blocks, masks, p)
            ref = oracle.compress_blocks(fmt, blocks, masks, oracle.make_params(alg, weights, aw))
            check_blocks(oracle, fmt, got, ref, blocks, masks, weights, alg != 0,
                         "adversarial %s alg%d aw%d" % (FMT_NAMES[fmt], alg, aw))


@pytest.mark.parametrize("fmt,alg", [(0, 1), (0, 0), (2, 1), (2, 2), (1, 0), (3, 1), (4, 1)])
def test_every_mask(tx, cuda, oracle, fmt, alg):
    base = workloads.random_blocks(8, seed=55)
    sel = base[[3, 5, 6]]
    blocks = np.repeat(sel, 1 << 16, axis=0)
    masks = np.tile(np.arange(1 << 16, dtype=np.uint32), sel.shape[0])
    p = tx_params(tx, alg)
    got = dev_compress_blocks(tx, cuda, fmt, blocks, masks, p)
    ref = oracle.compress_blocks(fmt, blocks, masks, oracle.make_params(alg))
    check_blocks(oracle, fmt, got, ref, blocks, masks, PERCEPTUAL, alg != 0,
                 "every mask %s alg%d" % (FMT_NAMES[fmt], alg))


def test_odd_sizes_and_extra_rows(tx, cuda, oracle):
    rng = np.random.default_rng(9)
    for w in range(1, 10):
        for h in range(0, 10):
            img = rng.integers(0, 256, size=(h, w, 4), dtype=np.uint8)
            for fmt in range(5):
                f = tx.Format(fmt)
                bs = f.block_size()
                extra = int(rng.integers(0, 3)) * tx.num_blocks(w) * bs + int(rng.integers(0, 2)) * bs
                n = f.compressed_size(w, h) + extra
                alg = int(rng.integers(0, 3))
                p = tx_params(tx, alg)
                got = np.zeros(n, np.uint8)
                f.compress(img, w, h, p, got)
                ref = oracle.compress(fmt, img, w, h, oracle.make_params(alg), out_len=n)
                if not np.array_equal(got, ref):
                    blocks, masks = workloads.image_to_blocks(img) if h else (None, None)
                    assert alg != 0 and blocks is not None, (w, h, fmt, alg, n)
                    k = blocks.shape[0]
                    check_blocks(oracle, fmt, got[:k * bs].reshape(k, bs), ref[:k * bs].reshape(k, bs),
                                 blocks, masks, PERCEPTUAL, True, "odd %dx%d" % (w, h))
                    assert np.array_equal(got[k * bs:], ref[k * bs:])


def test_unaligned_pitch_and_native_paths(tx, cuda, oracle):
    # widths whose rows are not 16-byte aligned take the per-pixel load path
    for w, h in ((37, 29), (130, 66), (4, 1025)):
        img = workloads.ramp_texture(w, h, seed=w, alpha="ramp")
        compare_image(tx, cuda, oracle, 2, img, 1, label="pitch %dx%d" % (w, h))
        compare_image(tx, cuda, oracle, 0, img, 0, label="pitch %dx%d range" % (w, h))
        r = workloads.value_noise(w, h, channels=2, seed=w)
        rgba = workloads.expand_to_rgba(r)
        for fmt, ch in ((3, 1), (4, 2)):
            ref = oracle.compress(fmt, rgba, w, h, oracle.make_params())
            got = dev_compress(tx, cuda, fmt, np.ascontiguousarray(r[..., :ch]), tx.Params(), channels=ch)
            assert np.array_equal(got, ref), (fmt, w, h)


def test_decoders_match_oracle(tx, cuda, oracle):
    rng = np.random.default_rng(4)
    for fmt in range(5):
        f = tx.Format(fmt)
        bs = f.block_size()
        w, h = 37, 23
        data = rng.integers(0, 256, size=f.compressed_size(w, h), dtype=np.uint8)
        out = np.zeros(w * h * 4, np.uint8)
        f.decompress(data, w, h, out)
        ref = oracle.decompress(fmt, data, w, h)
        assert np.array_equal(out, ref), FMT_NAMES[fmt]
        for b in range(0, data.size // bs, 17):
            assert np.array_equal(np.frombuffer(f.decompress_block(data[b * bs:(b + 1) * bs]), np.uint8),
                                  oracle.decompress_block(fmt, data[b * bs:(b + 1) * bs]))


def test_large_textures(tx, cuda, oracle):
    """~134 M pixels with sides that are not multiples of 4: 32-bit block
    counts, grid sizing and the last partial block row and column."""
    w, h = 16382, 8193
    rng = np.random.default_rng(12)
    # RangeFit BC1 on a tiled noisy ramp texture
    tile = workloads.ramp_texture(1024, 1024, seed=13)
    rgba = np.ascontiguousarray(np.tile(tile, (9, 17, 1))[:h, :w])
    rgba[rng.integers(0, h, 64), rng.integers(0, w, 64), 3] = 0  # a few transparent pixels
    p = tx_params(tx, 0)
    got = dev_compress(tx, cuda, 0, rgba, p)
    ref = oracle.compress(0, rgba, w, h, oracle.make_params(0, PERCEPTUAL, False))
    assert np.array_equal(got, ref), "BC1 RangeFit %dx%d differs" % (w, h)
    del rgba, got, ref
    # BC4 from native R8
    r8 = np.ascontiguousarray(np.tile(workloads.value_noise(1024, 1024, channels=1, seed=14), (9, 17, 1))[:h, :w])
    got = dev_compress(tx, cuda, 3, r8, tx.Params(), channels=1)
    ref = oracle.compress(3, workloads.expand_to_rgba(r8), w, h, oracle.make_params())
    assert np.array_equal(got, ref), "BC4 R8 %dx%d differs" % (w, h)
