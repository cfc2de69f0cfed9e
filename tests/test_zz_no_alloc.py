"""tx_batch_launch_noalloc: the allocation-free batch launch for callers that
must not have the library allocate device memory (fixed memory budgets owned
by the caller's allocator, frame loops that cannot absorb an allocation's
implicit synchronisation).  Its work queue lives in a fixed device array, so
its bytes must equal those of the existing per-level entry point
(tx_compress_device), call after call, while the array is reused.

This file is collected last on purpose; it also passes alone in a fresh
process."""
import ctypes

import numpy as np
import pytest

from texpresso_gb300 import workloads

pytestmark = pytest.mark.gpu


def _noalloc(tx):
    lib = tx.library()
    f = lib.tx_batch_launch_noalloc
    f.argtypes = [ctypes.POINTER(tx.BatchItem), ctypes.c_size_t, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _levels(torch, tx, seed, n):
    """n texture levels of mixed formats, algorithms, sizes and channel layouts."""
    rng = np.random.default_rng(seed)
    srcs, outs, items, per_call = [], [], [], []
    for i in range(n):
        fmt = int(rng.integers(0, 5))
        alg = int(rng.integers(0, 3))
        w, h = int(rng.integers(1, 150)), int(rng.integers(1, 150))
        ch = 4
        if fmt == 3 and rng.integers(0, 2):
            ch = 1
        if fmt == 4 and rng.integers(0, 2):
            ch = 2
        img = workloads.ramp_texture(w, h, seed=seed * 1000 + i, alpha="ramp")
        if ch < 4:
            img = np.ascontiguousarray(img[..., :ch])
        p = tx.Params(algorithm=tx.Algorithm(alg), weigh_colour_by_alpha=bool(rng.integers(0, 2)))
        t = torch.from_numpy(img).cuda()
        n_out = tx.Format(fmt).compressed_size(w, h)
        o = torch.zeros(n_out, dtype=torch.uint8, device="cuda")
        r = torch.zeros(n_out, dtype=torch.uint8, device="cuda")
        tx.compress_device(tx.Format(fmt), t.data_ptr(), w * ch, ch, w, h, p, r.data_ptr(), n_out,
                           torch.cuda.current_stream().cuda_stream)
        srcs.append(t)
        outs.append(o)
        per_call.append(r)
        items.append(tx.batch_item(fmt, t.data_ptr(), w * ch, w, h, p, o.data_ptr(), channels=ch))
    torch.cuda.synchronize()
    return srcs, outs, items, [r.cpu().numpy() for r in per_call]


def test_noalloc_matches_existing_entry_point_twice(tx, cuda):
    torch = cuda
    launch = _noalloc(tx)
    stream = torch.cuda.current_stream().cuda_stream
    for call, (seed, n) in enumerate(((1, 40), (2, 25))):
        srcs, outs, items, ref = _levels(torch, tx, seed, n)
        arr = (tx.BatchItem * n)(*items)
        rc = launch(arr, n, stream)
        assert rc == 0, tx.TexpressoError(rc, "tx_batch_launch_noalloc")
        torch.cuda.synchronize()
        for k, (o, r) in enumerate(zip(outs, ref)):
            assert np.array_equal(o.cpu().numpy(), r), "call %d, item %d differs" % (call, k)
        del srcs


def _flat_blocks_texture(torch, width, height, seed, noisy_every=64):
    """RGBA8 on the device: one random colour per 4x4 block (the single-colour
    path), every `noisy_every`-th block a noisy ramp instead (full ClusterFit)."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    bw, bh = width // 4, height // 4
    col = torch.randint(0, 256, (bh, bw, 4), generator=g, device="cuda", dtype=torch.uint8)
    col[..., 3] = 255
    img = col.repeat_interleave(4, 0).repeat_interleave(4, 1).contiguous()
    noise = torch.randint(0, 256, (height, width, 3), generator=g, device="cuda", dtype=torch.uint8)
    sel = torch.zeros((bh, bw), dtype=torch.bool, device="cuda")
    sel.view(-1)[::noisy_every] = True
    sel = sel.repeat_interleave(4, 0).repeat_interleave(4, 1)
    img[..., :3] = torch.where(sel[..., None], noise, img[..., :3])
    return img


def test_noalloc_large_levels_grow_the_units(tx, cuda):
    """Levels large enough that the default units overflow the fixed array:
    the team units grow past 64 blocks (an 8.4 M-block BC1 ClusterFit level)
    and the lane units past 64 blocks (8192x8192 BC4 R8 and BC5 RG8), with an
    IterativeClusterFit level drained by the prefetching team kernel at the
    grown unit size.  Bytes must still equal the per-level entry point's, on
    two calls in a row."""
    torch = cuda
    launch = _noalloc(tx)
    stream = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device="cuda").manual_seed(5)
    C = tx.Algorithm.ClusterFit
    levels = [
        (0, 16384, 8192, 4, tx.Params(algorithm=C), _flat_blocks_texture(torch, 16384, 8192, 1)),
        (3, 8192, 8192, 1, tx.Params(),
         torch.randint(0, 256, (8192, 8192, 1), generator=g, device="cuda", dtype=torch.uint8)),
        (4, 8192, 8192, 2, tx.Params(),
         torch.randint(0, 256, (8192, 8192, 2), generator=g, device="cuda", dtype=torch.uint8)),
        (2, 1024, 1024, 4, tx.Params(algorithm=tx.Algorithm.IterativeClusterFit),
         torch.from_numpy(workloads.ramp_texture(1024, 1024, seed=6, alpha="ramp")).cuda()),
        (2, 516, 509, 4, tx.Params(algorithm=C, weigh_colour_by_alpha=True),
         torch.from_numpy(workloads.ramp_texture(516, 509, seed=7, alpha="ramp")).cuda()),
    ]
    ref, items, outs = [], [], []
    for fmt, w, h, ch, p, img in levels:
        n_out = tx.Format(fmt).compressed_size(w, h)
        r = torch.zeros(n_out, dtype=torch.uint8, device="cuda")
        tx.compress_device(tx.Format(fmt), img.data_ptr(), w * ch, ch, w, h, p, r.data_ptr(), n_out, stream)
        ref.append(r)
        o = torch.zeros(n_out, dtype=torch.uint8, device="cuda")
        outs.append(o)
        items.append(tx.batch_item(fmt, img.data_ptr(), w * ch, w, h, p, o.data_ptr(), channels=ch))
    arr = (tx.BatchItem * len(items))(*items)
    for call in range(2):
        for o in outs:
            o.fill_(0xA5)
        rc = launch(arr, len(items), stream)
        assert rc == 0, tx.TexpressoError(rc, "tx_batch_launch_noalloc")
        torch.cuda.synchronize()
        for k, (o, r) in enumerate(zip(outs, ref)):
            assert torch.equal(o, r), "call %d, level %d differs in %d bytes" % (
                call, k, int((o != r).sum()))


def test_noalloc_rejects_more_items_than_the_array_holds(tx, cuda):
    torch = cuda
    launch = _noalloc(tx)
    src = torch.zeros(64, dtype=torch.uint8, device="cuda")
    dst = torch.zeros(16, dtype=torch.uint8, device="cuda")
    item = tx.batch_item(0, src.data_ptr(), 16, 4, 4, tx.Params(), dst.data_ptr())
    arr = (tx.BatchItem * 257)(*([item] * 257))
    assert launch(arr, 257, torch.cuda.current_stream().cuda_stream) == -2
    assert launch(arr, 256, torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
