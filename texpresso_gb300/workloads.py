"""Seeded synthetic textures with the shapes and value distributions of the
benchmark configurations (the reference publishes no benchmark data, so these
generators stand in for it).

* ``ramp_texture``   -- per 4x4 block a two-endpoint linear colour ramp along a
  random direction plus Gaussian noise (sigma 6), clamped to u8, alpha 255;
  a fraction of blocks is a single flat colour.  Optional per-block alpha
  ramp with uniform noise and forced 0/255 extremes in some blocks.
* ``value_noise``    -- a smooth multi-octave value-noise field quantised to u8
  with uniform dither, one or two channels (BC4 / BC5 inputs).
* ``random_blocks``  -- adversarial single blocks for edge-case testing.
* ``grid_blocks``    -- blocks whose colours lie on the 5:6:5 endpoint grid.

All functions are pure numpy and deterministic for a given seed.
"""
import numpy as np


def ramp_texture(width, height, seed=0, flat_frac=0.10, sigma=6.0, alpha="opaque",
                 alpha_noise=12, extreme_frac=0.15):
    """RGBA8 image (height, width, 4) of per-block noisy linear ramps.

    alpha: "opaque" (255 everywhere) or "ramp" (per-block random u8 ramp plus
    uniform noise in [-alpha_noise, alpha_noise]; extreme_frac of the blocks
    get one pixel forced to 0 and one to 255).
    """
    rng = np.random.default_rng(seed)
    bw, bh = (width + 3) // 4, (height + 3) // 4
    nb = bw * bh
    c0 = rng.uniform(0, 255, size=(nb, 1, 3))
    c1 = rng.uniform(0, 255, size=(nb, 1, 3))
    t = rng.uniform(0, 1, size=(nb, 16, 1))
    col = c0 + t * (c1 - c0) + rng.normal(0.0, sigma, size=(nb, 16, 3))
    flat = rng.uniform(0, 1, size=nb) < flat_frac
    col[flat] = rng.uniform(0, 255, size=(int(flat.sum()), 1, 3))
    col = np.clip(np.rint(col), 0, 255).astype(np.uint8)
    if alpha == "opaque":
        a = np.full((nb, 16, 1), 255, np.uint8)
    else:
        a0 = rng.uniform(0, 255, size=(nb, 1))
        a1 = rng.uniform(0, 255, size=(nb, 1))
        pos = (np.arange(16) % 4 + np.arange(16) // 4) / 6.0
        av = a0 + (a1 - a0) * pos[None, :] + rng.integers(-alpha_noise, alpha_noise + 1, size=(nb, 16))
        ext = rng.uniform(0, 1, size=nb) < extreme_frac
        idx = np.flatnonzero(ext)
        p0 = rng.integers(0, 16, size=idx.size)
        p1 = (p0 + rng.integers(1, 16, size=idx.size)) % 16
        av[idx, p0] = 0
        av[idx, p1] = 255
        a = np.clip(np.rint(av), 0, 255).astype(np.uint8)[..., None]
    blocks = np.concatenate([col, a], axis=2).reshape(bh, bw, 4, 4, 4)
    img = blocks.transpose(0, 2, 1, 3, 4).reshape(bh * 4, bw * 4, 4)
    return np.ascontiguousarray(img[:height, :width])


def value_noise(width, height, channels=1, seed=0, octaves=8, dither=3):
    """u8 image (height, width, channels): multi-octave value noise + dither.

    Octave o is a (4*2^o + 1)^2 lattice of uniform values, smoothstep-
    interpolated (separably: along x, then along y) and weighted 0.5^o."""
    rng = np.random.default_rng(seed)
    out = np.zeros((height, width, channels), np.float32)
    ys = (np.arange(height, dtype=np.float32) + 0.5) / height
    xs = (np.arange(width, dtype=np.float32) + 0.5) / width
    total = 0.0
    for o in range(octaves):
        cells = 4 << o
        amp = np.float32(0.5 ** o)
        total += float(amp)
        grid = rng.uniform(0, 1, size=(cells + 1, cells + 1, channels)).astype(np.float32)
        gy, gx = ys * cells, xs * cells
        iy = np.minimum(gy.astype(np.int64), cells - 1)
        ix = np.minimum(gx.astype(np.int64), cells - 1)
        fy = (gy - iy).astype(np.float32)
        fx = (gx - ix).astype(np.float32)
        fy = (fy * fy * (3 - 2 * fy))[:, None, None]
        fx = (fx * fx * (3 - 2 * fx))[None, :, None]
        rows = grid[:, ix] * (1 - fx) + grid[:, ix + 1] * fx      # (cells+1, width, ch)
        out += amp * (rows[iy] * (1 - fy) + rows[iy + 1] * fy)
    out *= np.float32(255.0 / total)
    out += rng.integers(-dither, dither + 1, size=out.shape, dtype=np.int8).astype(np.float32)
    return np.clip(np.rint(out), 0, 255).astype(np.uint8)


def expand_to_rgba(img):
    """R8 / RG8 -> RGBA8 with the other channels 0 and alpha 255 (the layout the
    reference's compress reads for BC4 / BC5, lib/src/lib.rs:323)."""
    h, w, c = img.shape
    out = np.zeros((h, w, 4), np.uint8)
    out[..., :c] = img
    out[..., 3] = 255
    return out


def image_to_blocks(img):
    """RGBA8 (h, w, 4) -> (nblocks, 64) blocks and (nblocks,) masks, block-row order."""
    h, w, _ = img.shape
    bw, bh = (w + 3) // 4, (h + 3) // 4
    pad = np.zeros((bh * 4, bw * 4, 4), np.uint8)
    pad[:h, :w] = img
    valid = np.zeros((bh * 4, bw * 4), bool)
    valid[:h, :w] = True
    blocks = pad.reshape(bh, 4, bw, 4, 4).transpose(0, 2, 1, 3, 4).reshape(-1, 64)
    v = valid.reshape(bh, 4, bw, 4).transpose(0, 2, 1, 3).reshape(-1, 16)
    masks = (v.astype(np.uint32) << np.arange(16, dtype=np.uint32)).sum(axis=1).astype(np.uint32)
    return np.ascontiguousarray(blocks), masks


def random_blocks(n, seed=0):
    """(n, 64) RGBA8 blocks mixing the shapes that drive different code paths:
    flat, two-colour, few colours with duplicates, noisy ramps, colours varying
    only along (1,-1,0) (degenerate principal axis), transparent pixels, alpha
    extremes."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 16, 4), np.uint8)
    kind = rng.integers(0, 8, size=n)
    for b in range(n):
        k = kind[b]
        if k == 0:
            out[b, :, :] = rng.integers(0, 256, size=4)
        elif k == 1:
            cols = rng.integers(0, 256, size=(2, 4))
            out[b] = cols[rng.integers(0, 2, size=16)]
        elif k == 2:
            cols = rng.integers(0, 256, size=(rng.integers(2, 6), 4))
            out[b] = cols[rng.integers(0, len(cols), size=16)]
        elif k == 3:
            c0, c1 = rng.uniform(0, 255, size=(2, 4))
            t = rng.uniform(0, 1, size=(16, 1))
            out[b] = np.clip(np.rint(c0 + t * (c1 - c0) + rng.normal(0, 6, size=(16, 4))), 0, 255)
        elif k == 4:
            base = rng.integers(40, 216)
            d = rng.integers(-40, 41, size=16)
            out[b, :, 0] = base + d
            out[b, :, 1] = base - d
            out[b, :, 2] = rng.integers(0, 256)
            out[b, :, 3] = 255
        elif k == 5:
            out[b] = rng.integers(0, 256, size=(16, 4))
        elif k == 6:
            out[b] = rng.integers(0, 256, size=(16, 4))
            out[b, rng.integers(0, 16, size=3), 3] = rng.choice([0, 255], size=3)
        else:
            v = rng.integers(0, 256, size=(16, 4))
            v[:, 3] = rng.choice([0, 127, 128, 255], size=16)
            out[b] = v
    return out.reshape(n, 64)


# ---------------------------------------------------------------------------
# batched configuration: many textures of uneven sizes with mip chains

def batch_specs(n=1000, seed=0, min_side=4, max_side=4096, formats=(0, 2, 4), algorithms=(0, 1, 2)):
    """Texture specs: width and height log-uniform in [min_side, max_side]
    (non-multiples of 4 allowed), format and algorithm drawn uniformly."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(min_side), np.log(max_side + 1)
    ws = np.floor(np.exp(rng.uniform(lo, hi, n))).astype(int).clip(min_side, max_side)
    hs = np.floor(np.exp(rng.uniform(lo, hi, n))).astype(int).clip(min_side, max_side)
    fm = rng.choice(formats, n)
    al = rng.choice(algorithms, n)
    return [{"width": int(w), "height": int(h), "format": int(f), "algorithm": int(a), "seed": int(seed * 100003 + i)}
            for i, (w, h, f, a) in enumerate(zip(ws, hs, fm, al))]


def ramp_texture_torch(width, height, seed, device, flat_frac=0.10, sigma=6.0, alpha="ramp"):
    """ramp_texture's distribution generated with torch on `device` (fast for
    large batches; the values differ from the numpy generator's)."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    bw, bh = (width + 3) // 4, (height + 3) // 4
    nb = bw * bh
    u = lambda *s: torch.rand(*s, generator=g, device=device)
    c0 = u(nb, 1, 3) * 255
    c1 = u(nb, 1, 3) * 255
    col = c0 + u(nb, 16, 1) * (c1 - c0) + torch.randn(nb, 16, 3, generator=g, device=device) * sigma
    flat = u(nb) < flat_frac
    col = torch.where(flat[:, None, None], c0.expand(nb, 16, 3), col)
    col = col.round().clamp(0, 255).to(torch.uint8)
    if alpha == "ramp":
        a0, a1 = u(nb, 1) * 255, u(nb, 1) * 255
        pos = ((torch.arange(16, device=device) % 4 + torch.arange(16, device=device) // 4) / 6.0)[None, :]
        av = a0 + (a1 - a0) * pos + torch.randint(-12, 13, (nb, 16), generator=g, device=device)
        a = av.round().clamp(0, 255).to(torch.uint8)[..., None]
    else:
        a = torch.full((nb, 16, 1), 255, dtype=torch.uint8, device=device)
    blocks = torch.cat([col, a], dim=2).reshape(bh, bw, 4, 4, 4)
    img = blocks.permute(0, 2, 1, 3, 4).reshape(bh * 4, bw * 4, 4)
    return img[:height, :width].contiguous()


def mip_reference(img):
    """Next mip level of an (h, w, c) u8 image with the library's box filter:
    (a+b+c+d+2)>>2 over the 2x2 source footprint, coordinates clamped."""
    h, w, c = img.shape
    dw, dh = max(1, w // 2), max(1, h // 2)
    xs0 = np.minimum(2 * np.arange(dw), w - 1)
    xs1 = np.minimum(2 * np.arange(dw) + 1, w - 1)
    ys0 = np.minimum(2 * np.arange(dh), h - 1)
    ys1 = np.minimum(2 * np.arange(dh) + 1, h - 1)
    s = (img[ys0][:, xs0].astype(np.uint32) + img[ys0][:, xs1] + img[ys1][:, xs0] + img[ys1][:, xs1])
    return ((s + 2) >> 2).astype(np.uint8)


def grid_blocks(n, seed):
    """Blocks whose colours are 5:6:5 grid values: 2-4 palette entries, or 16
    entries one grid step apart."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 16, 4), np.uint8)
    for b in range(n):
        k = int(rng.integers(2, 5))
        pal = np.stack([rng.integers(0, 32, k) * 255 // 31, rng.integers(0, 64, k) * 255 // 63,
                        rng.integers(0, 32, k) * 255 // 31, rng.integers(0, 256, k)], 1)
        blk = pal[rng.integers(0, k, 16)]
        if b % 3 == 0:
            base = np.array([rng.integers(0, 28), rng.integers(0, 60), rng.integers(0, 28)])
            steps = np.stack([(base[0] + np.arange(16) % 4), (base[1] + np.arange(16) // 4),
                              (base[2] + (np.arange(16) % 3))], 1)
            blk[:, 0] = steps[:, 0] * 255 // 31
            blk[:, 1] = steps[:, 1] * 255 // 63
            blk[:, 2] = steps[:, 2] * 255 // 31
        out[b] = blk
    return out.reshape(n, 64)
