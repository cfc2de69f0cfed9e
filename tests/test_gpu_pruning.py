"""ClusterFit candidate pruning is exact: with the error lower bound the GPU
skips candidates, and the packed output must still equal the oracle's (which
evaluates every candidate) bit for bit, with no tie allowance.  The blocks and
weights aim at the bound's margin: colours on the 5:6:5 grid (snapped and
unsnapped optimum coincide), few distinct colours (near-singular systems,
duplicate weights), alpha weighting, zero, subnormal, huge, negative and
non-finite channel weights (the last two must fall back to the plain sweep)."""
import numpy as np
import pytest

from texpresso_gb300 import workloads

pytestmark = pytest.mark.gpu

WEIGHT_SETS = [
    (0.2126, 0.7152, 0.0722), (1.0, 1.0, 1.0), (1.0, 0.0, 0.0), (0.0, 0.0, 0.0), (1e-40, 1.0, 1e-3),
    (1e6, 1e6, 1e6), (3e38, 1.0, 1.0), (-1.0, 1.0, 1.0), (float("inf"), 1.0, 1.0), (float("nan"), 1.0, 1.0),
]


def dev_compress_blocks(tx, torch, fmt, blocks, params):
    b = torch.from_numpy(np.ascontiguousarray(blocks)).cuda()
    f = tx.Format(fmt)
    out = torch.zeros(blocks.shape[0] * f.block_size(), dtype=torch.uint8, device="cuda")
    tx.compress_blocks_device(f, b.data_ptr(), 0, blocks.shape[0], params, out.data_ptr(),
                              torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(blocks.shape[0], -1)


@pytest.mark.parametrize("fmt", [0, 2])
@pytest.mark.parametrize("alg", [1, 2])
def test_pruned_clusterfit_bit_exact(tx, cuda, oracle, fmt, alg):
    blocks = np.concatenate([workloads.random_blocks(1500, seed=300 + fmt), workloads.grid_blocks(1500, seed=400 + fmt),
                             workloads.image_to_blocks(workloads.ramp_texture(128, 128, seed=5 + fmt,
                                                                              alpha="ramp"))[0]])
    for weights in WEIGHT_SETS:
        for aw in (False, True):
            p = tx.Params(algorithm=tx.Algorithm(alg), weights=weights, weigh_colour_by_alpha=aw)
            got = dev_compress_blocks(tx, cuda, fmt, blocks, p)
            ref = oracle.compress_blocks(fmt, blocks, None, oracle.make_params(alg, weights, aw))
            diff = np.flatnonzero(np.any(got != ref, axis=1))
            assert diff.size == 0, "fmt %d alg %d weights %r aw %d: %d blocks differ (first %d)" % (
                fmt, alg, weights, aw, diff.size, diff[0])


def flat_noise_blocks(n, seed, spread=3):
    """Nearly flat 16-colour blocks (one colour plus small per-pixel noise):
    their candidates' errors lie within the bound's margin of one another,
    so most of them survive the bound and the exact sweep is long."""
    rng = np.random.default_rng(seed)
    base = rng.integers(24, 232, size=(n, 1, 3))
    col = np.clip(base + rng.integers(-spread, spread + 1, size=(n, 16, 3)), 0, 255).astype(np.uint8)
    a = rng.integers(0, 256, size=(n, 16, 1)).astype(np.uint8)
    return np.concatenate([col, a], axis=2).reshape(n, 64)


@pytest.mark.parametrize("fmt", [0, 2])
def test_long_survivor_queues_bit_exact(tx, cuda, oracle, fmt):
    """Nearly flat blocks (hundreds of survivors each) mixed with ordinary and
    adversarial ones in a launch of more than one wave, which runs in 8-team
    CTAs (the smaller launches above run in one-warp CTAs): bit for bit equal
    to the oracle."""
    blocks = np.concatenate([flat_noise_blocks(3000, seed=700 + fmt),
                             workloads.image_to_blocks(workloads.ramp_texture(256, 256, seed=9 + fmt,
                                                                              alpha="ramp"))[0],
                             workloads.random_blocks(1000, seed=710 + fmt)])
    assert blocks.shape[0] > 152 * 4 * 8  # more than one wave of 8-team CTAs on a GB300
    for weights in [(0.2126, 0.7152, 0.0722), (1.0, 1.0, 1.0), (1.0, 0.0, 0.0), (1e6, 1e6, 1e6)]:
        for aw in (False, True):
            p = tx.Params(algorithm=tx.Algorithm(1), weights=weights, weigh_colour_by_alpha=aw)
            got = dev_compress_blocks(tx, cuda, fmt, blocks, p)
            ref = oracle.compress_blocks(fmt, blocks, None, oracle.make_params(1, weights, aw))
            diff = np.flatnonzero(np.any(got != ref, axis=1))
            assert diff.size == 0, "fmt %d weights %r aw %d: %d blocks differ (first %d)" % (
                fmt, weights, aw, diff.size, diff[0])
