"""The batched form (tx_batch_*): many texture levels of mixed formats and
algorithms in one launch must produce exactly the bytes of one
tx_compress_device call per level, and those bytes must equal the oracle's.
Also the mip producer against its numpy definition, CUDA-graph replay,
launch-shape tuning and the autotuner."""
import numpy as np
import pytest

from texpresso_gb300 import workloads

pytestmark = pytest.mark.gpu


def _specs(n, seed, max_side=260):
    rng = np.random.default_rng(seed)
    specs = workloads.batch_specs(n, seed=seed, min_side=1, max_side=max_side, formats=(0, 1, 2, 3, 4))
    for s in specs:
        s["aw"] = bool(rng.integers(0, 2))
    return specs


@pytest.fixture(scope="module")
def tset(tx, cuda):
    from texpresso_gb300.texture_set import TextureSet
    return TextureSet(_specs(48, seed=5), device="cuda")


def test_mips_match_definition(tx, cuda, tset):
    for lv in tset.levels[:20]:
        imgs = [l.cpu().numpy() for l in lv]
        assert imgs[-1].shape[:2] == (1, 1)
        assert len(imgs) == tx.mip_count(imgs[0].shape[1], imgs[0].shape[0])
        for a, b in zip(imgs[:-1], imgs[1:]):
            assert np.array_equal(workloads.mip_reference(a), b)


def test_batch_equals_per_call_and_oracle(tx, cuda, tset, oracle):
    from texpresso_gb300.texture_set import same
    st = cuda.cuda.current_stream().cuda_stream
    tset.per_call(st)
    cuda.cuda.synchronize()
    ref = tset.snapshot()
    tset.clear_outputs()
    b = tx.Batch(tset.items())
    b.launch(st)
    cuda.cuda.synchronize()
    got = tset.snapshot()
    assert same(got, ref)
    # oracle on every level of a handful of textures
    for i in range(0, len(tset.specs), 5):
        s = tset.specs[i]
        for lvl, img in enumerate(l.cpu().numpy() for l in tset.levels[i]):
            h, w = img.shape[:2]
            o = oracle.compress(s["format"], img, w, h, oracle.make_params(s["algorithm"], (0.2126, 0.7152, 0.0722),
                                                                           s["aw"]))
            assert np.array_equal(got[i][lvl], o), (i, lvl, s)
    b.close()


@pytest.mark.parametrize("tuning", [
    dict(team_lanes=16, team_threads_per_cta=128, team_ctas_per_sm=2, team_blocks_per_unit=3,
         lane_ctas_per_sm=2, lane_blocks_per_lane=1, team_blocks_in_flight=1),
    dict(team_lanes=32, team_threads_per_cta=64, team_ctas_per_sm=1, team_blocks_per_unit=8,
         lane_ctas_per_sm=6, lane_blocks_per_lane=8, team_blocks_in_flight=3),
    dict(team_lanes=32, team_threads_per_cta=256, team_ctas_per_sm=4, team_blocks_per_unit=5,
         lane_ctas_per_sm=3, lane_blocks_per_lane=2, team_blocks_in_flight=2),
    dict(team_lanes=16, team_threads_per_cta=256, team_ctas_per_sm=3, team_blocks_per_unit=1,
         lane_ctas_per_sm=4, lane_blocks_per_lane=3, team_blocks_in_flight=3),
])
def test_launch_shapes_do_not_change_bytes(tx, cuda, tset, tuning):
    from texpresso_gb300.texture_set import same
    st = cuda.cuda.current_stream().cuda_stream
    b = tx.Batch(tset.items())
    b.launch(st)
    cuda.cuda.synchronize()
    ref = tset.snapshot()
    t = tx.BatchTuning(**tuning)
    b.tuning = t
    assert b.tuning.as_dict() == t.as_dict()
    tset.clear_outputs()
    b.launch(st)
    cuda.cuda.synchronize()
    assert same(tset.snapshot(), ref)
    b.close()


def test_graph_replay_and_autotune(tx, cuda, tset):
    from texpresso_gb300.texture_set import same
    torch = cuda
    b = tx.Batch(tset.items())
    s = torch.cuda.Stream()
    b.launch(s.cuda_stream)
    torch.cuda.synchronize()
    ref = tset.snapshot()
    chosen = b.autotune(s.cuda_stream, repeats=1)
    assert chosen.team_lanes in (16, 32)
    tset.clear_outputs()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.launch(s.cuda_stream)
    for _ in range(2):
        tset.clear_outputs()
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        assert same(tset.snapshot(), ref)
    info = b.info()
    assert info["blocks"] == tset.blocks() and info["lane_units"] + info["team_units"] > 0
    b.close()


def test_native_channel_items(tx, cuda, oracle):
    torch = cuda
    r = workloads.value_noise(70, 45, channels=2, seed=8)
    rgba = workloads.expand_to_rgba(r)
    srcs, outs, items = [], [], []
    for fmt, ch in ((3, 1), (4, 2), (3, 4), (4, 4)):
        img = np.ascontiguousarray(r[..., :ch]) if ch < 4 else rgba
        t = torch.from_numpy(img).cuda()
        o = torch.zeros(tx.Format(fmt).compressed_size(70, 45), dtype=torch.uint8, device="cuda")
        srcs.append(t)
        outs.append(o)
        items.append(tx.batch_item(fmt, t.data_ptr(), 70 * ch, 70, 45, tx.Params(), o.data_ptr(), channels=ch))
    b = tx.Batch(items)
    b.launch(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for (fmt, ch), o in zip(((3, 1), (4, 2), (3, 4), (4, 4)), outs):
        assert np.array_equal(o.cpu().numpy(), oracle.compress(fmt, rgba, 70, 45, oracle.make_params())), (fmt, ch)
    b.close()


def test_config3_textures_match_oracle(tx, cuda, oracle):
    """Thirty textures of the benchmark's own 1,000-texture batch
    (batch_specs(1000, seed=0), the same content generator): the largest of
    every format x algorithm class (up to 3880x2918) and 21 others drawn at
    random, every mip level compressed by one batch launch and compared with
    the oracle's compress of that level (lib/src/lib.rs:287-335), bit for bit."""
    from texpresso_gb300.texture_set import TextureSet
    specs = workloads.batch_specs(1000, seed=0)
    largest = {}
    for i, s in enumerate(specs):
        k = (s["format"], s["algorithm"])
        if k not in largest or s["width"] * s["height"] > specs[largest[k]]["width"] * specs[largest[k]]["height"]:
            largest[k] = i
    assert len(largest) == 9
    rest = [i for i in range(len(specs)) if i not in set(largest.values())]
    pick = sorted(set(largest.values()) | set(np.random.default_rng(1).choice(rest, 21, replace=False).tolist()))
    chosen = [specs[i] for i in pick]
    ts = TextureSet(chosen, device="cuda")
    st = cuda.cuda.current_stream().cuda_stream
    b = tx.Batch(ts.items())
    b.launch(st)
    cuda.cuda.synchronize()
    got = ts.snapshot()
    b.close()
    levels = blocks = 0
    for i, s in enumerate(chosen):
        op = oracle.make_params(s["algorithm"], (0.2126, 0.7152, 0.0722), False)
        for lvl, img in enumerate(l.cpu().numpy() for l in ts.levels[i]):
            h, w = img.shape[:2]
            ref = oracle.compress(s["format"], img, w, h, op)
            assert np.array_equal(got[i][lvl], ref), "texture %d (%dx%d fmt %d alg %d) level %d differs" % (
                pick[i], s["width"], s["height"], s["format"], s["algorithm"], lvl)
            levels += 1
            blocks += tx.num_blocks(w) * tx.num_blocks(h)
    print("config-3 oracle check: %d textures, %d levels, %d blocks identical" % (len(chosen), levels, blocks))
