"""Device-resident textures with full mip chains, compressed either as one
batch (tx_batch_*) or one call per level (tx_compress_device).

torch provides device memory and streams; all pixel work (mip generation,
compression) runs in the library's kernels.
"""
import numpy as np

import texpresso_gb300 as tx
from texpresso_gb300 import workloads


class TextureSet:
    def __init__(self, specs, device="cuda", mips=True, stream=None, content=None):
        import torch
        self.torch = torch
        self.specs = specs
        self.device = torch.device(device)
        content = content or (lambda s: workloads.ramp_texture_torch(s["width"], s["height"], s["seed"], self.device))
        self.levels = []   # per texture: list of uint8 (h, w, 4) tensors, level 0 first
        for s in specs:
            self.levels.append([content(s)])
        if mips:
            self.build_mips(stream)
        self.outputs = [[torch.zeros(tx.Format(s["format"]).compressed_size(l.shape[1], l.shape[0]),
                                     dtype=torch.uint8, device=self.device) for l in lv]
                        for s, lv in zip(specs, self.levels)]

    def build_mips(self, stream=None):
        """Allocate every level and fill it with tx_mip_batch_device, one
        launch per level depth across all textures."""
        torch = self.torch
        depth = 0
        while True:
            jobs = []
            for lv in self.levels:
                src = lv[-1]
                h, w = src.shape[:2]
                if len(lv) != depth + 1 or (w == 1 and h == 1):
                    continue
                dst = torch.empty((max(1, h // 2), max(1, w // 2), 4), dtype=torch.uint8, device=self.device)
                lv.append(dst)
                jobs.append((src.data_ptr(), w * 4, w, h, 4, dst.data_ptr(), dst.shape[1] * 4))
            if not jobs:
                break
            tx.mip_batch_device(jobs, stream.cuda_stream if stream is not None else
                                torch.cuda.current_stream().cuda_stream)
            depth += 1

    def params(self, s):
        return tx.Params(algorithm=tx.Algorithm(s["algorithm"]), weigh_colour_by_alpha=s.get("aw", False))

    def items(self):
        out = []
        for s, lv, outs in zip(self.specs, self.levels, self.outputs):
            p = self.params(s)
            for img, o in zip(lv, outs):
                h, w = img.shape[:2]
                out.append(tx.batch_item(s["format"], img.data_ptr(), w * 4, w, h, p, o.data_ptr()))
        return out

    def blocks(self):
        return sum(tx.num_blocks(l.shape[1]) * tx.num_blocks(l.shape[0]) for lv in self.levels for l in lv)

    def pixels(self):
        return sum(l.shape[0] * l.shape[1] for lv in self.levels for l in lv)

    def per_call(self, stream):
        """The plain form: one tx_compress_device call per texture level."""
        for s, lv, outs in zip(self.specs, self.levels, self.outputs):
            p = self.params(s)
            f = tx.Format(s["format"])
            for img, o in zip(lv, outs):
                h, w = img.shape[:2]
                tx.compress_device(f, img.data_ptr(), w * 4, 4, w, h, p, o.data_ptr(), o.numel(), stream)

    def snapshot(self):
        return [[o.cpu().numpy().copy() for o in outs] for outs in self.outputs]

    def clear_outputs(self):
        for outs in self.outputs:
            for o in outs:
                o.zero_()


def level_images(ts, i):
    return [l.cpu().numpy() for l in ts.levels[i]]


def same(a, b):
    return all(np.array_equal(x, y) for xs, ys in zip(a, b) for x, y in zip(xs, ys))
