"""Replica sharding for N GPUs, exercised with world_size-2 gloo ranks on CPU.

Blocks are independent (lib/src/lib.rs:305-333), so ranks split work on the
host and exchange only timing: each rank owns a contiguous range of block
rows, and the reported time is the maximum over ranks."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, rows, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from texpresso_gb300 import replicas
    lo, hi = replicas.split_rows(rows, rank, world)
    t = replicas.max_over_ranks(1.5 + rank)
    replicas.barrier()
    q.put((rank, lo, hi, t))
    dist.destroy_process_group()


@pytest.mark.parametrize("rows", [1, 7, 512])
def test_two_rank_split_and_max(tx, rows):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, rows, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, lo0, hi0, t0), (r1, lo1, hi1, t1) = out
    assert lo0 == 0 and hi0 == lo1 and hi1 == rows
    assert abs((hi0 - lo0) - (hi1 - lo1)) <= 1
    assert t0 == t1 == 2.5
    del torch


def test_split_rows_tiles_exactly(tx):
    from texpresso_gb300 import replicas
    for world in (1, 2, 3, 8):
        for rows in (0, 1, 5, 100, 513):
            spans = [replicas.split_rows(rows, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == rows
            assert all(spans[i][1] == spans[i + 1][0] for i in range(world - 1))
