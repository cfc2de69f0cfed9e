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
