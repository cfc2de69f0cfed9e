"""The reference CLI's two flows (cli/src/main.rs:122-196) through this
library: PNG -> compress -> DDS, and DDS -> decompress -> PNG."""
import numpy as np
import pytest

from texpresso_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", [0, 1, 2, 3, 4])
def test_compress_then_decompress_files(tx, cuda, oracle, tmp_path, fmt):
    from texpresso_gb300 import pngio
    w, h = 45, 27
    img = workloads.ramp_texture(w, h, seed=fmt, alpha="ramp")
    src = str(tmp_path / "in.png")
    pngio.write_png(src, w, h, img)
    # compress_file: PNG -> RGBA8 -> Format::compress -> DDS
    ww, hh, rgba = pngio.read_png(src)
    f = tx.Format(fmt)
    blocks = np.zeros(f.compressed_size(ww, hh), np.uint8)
    f.compress(rgba, ww, hh, tx.Params(algorithm=tx.Algorithm.ClusterFit), blocks)
    dds = str(tmp_path / "out.dds")
    tx.write_dds(dds, f, ww, hh, blocks)
    # decompress_file: DDS -> Format::decompress -> PNG
    f2, w2, h2, _, data = tx.read_dds(dds)
    out = np.zeros(w2 * h2 * 4, np.uint8)
    f2.decompress(data, w2, h2, out)
    dst = str(tmp_path / "back.png")
    pngio.write_png(dst, w2, h2, out)
    _, _, back = pngio.read_png(dst)
    ref_blocks = oracle.compress(fmt, img, w, h, oracle.make_params(1))
    assert np.array_equal(blocks, ref_blocks)
    assert np.array_equal(back.reshape(-1), oracle.decompress(fmt, ref_blocks, w, h))
