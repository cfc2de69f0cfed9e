"""Multi-GPU replicas (no data-path collective).

4x4 blocks are independent (lib/src/lib.rs:305-333 keeps no state across
blocks), so several GPUs split work on the host -- whole textures or ranges of
block rows -- and concatenate outputs.  torch.distributed is used only to
line ranks up for timing and to take the maximum elapsed time.
"""
import os


def world():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def split_rows(rows, rank, world_size):
    """Contiguous [lo, hi) range of `rows` block rows owned by `rank`; ranges
    of consecutive ranks tile [0, rows) exactly and differ in size by <= 1."""
    base, extra = divmod(rows, world_size)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def max_over_ranks(value, device=None):
    """Maximum of a float over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(device=None):
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        if device is not None and dist.get_backend() == "nccl":
            dist.barrier(device_ids=[device.index if hasattr(device, "index") else int(device)])
        else:
            dist.barrier()
