"""Serving form (tx_server_*): jobs admitted by device memory, continuously
batched into shared compression steps.  Every job's bytes must equal the
oracle's per level, be the same alone and in a mix, and survive a budget
that forces jobs to queue for memory."""
import threading

import numpy as np
import pytest

from texpresso_gb300 import workloads

pytestmark = pytest.mark.gpu

PERCEPTUAL = (0.2126, 0.7152, 0.0722)


def _job(seed, side_max=300):
    rng = np.random.default_rng(seed)
    w, h = int(rng.integers(1, side_max)), int(rng.integers(1, side_max))
    fmt = int(rng.integers(0, 5))
    alg = int(rng.integers(0, 3))
    aw = bool(rng.integers(0, 2))
    mips = bool(rng.integers(0, 4))  # mostly with mips
    img = workloads.ramp_texture(w, h, seed=seed, alpha="ramp")
    return dict(img=img, w=w, h=h, fmt=fmt, alg=alg, aw=aw, mips=mips)


def _expected(oracle, j):
    out, img = [], j["img"]
    while True:
        h, w = img.shape[:2]
        out.append(oracle.compress(j["fmt"], img, w, h, oracle.make_params(j["alg"], PERCEPTUAL, j["aw"])))
        if not j["mips"] or (w == 1 and h == 1):
            break
        img = workloads.mip_reference(img)
    return np.concatenate(out)


def _submit(tx, srv, j):
    out = np.zeros(tx.chain_compressed_size(j["fmt"], j["w"], j["h"], j["mips"]), np.uint8)
    p = tx.Params(algorithm=tx.Algorithm(j["alg"]), weigh_colour_by_alpha=j["aw"])
    return srv.submit(j["img"], j["w"], j["h"], tx.Format(j["fmt"]), p, out, mips=j["mips"]), out


def test_jobs_match_oracle(tx, cuda, oracle):
    srv = tx.Server(memory_budget=256 << 20, step_blocks=4096, min_share=512)
    jobs = [_job(s) for s in range(40)]
    sub = [_submit(tx, srv, j) for j in jobs]
    for j, (rid, out) in zip(jobs, sub):
        res = srv.wait(rid, timeout_ms=60000)
        assert res["status"] == 0
        assert np.array_equal(out, _expected(oracle, j)), (j["w"], j["h"], j["fmt"], j["alg"], j["mips"])
    st = srv.stats()
    assert st["completed"] == 40 and st["steps"] > 0
    srv.close()


def test_same_alone_and_in_a_mix(tx, cuda):
    target = _job(1234, side_max=520)
    target["alg"], target["fmt"], target["mips"] = 2, 0, True  # iterative ClusterFit, BC1, mips
    srv = tx.Server(memory_budget=512 << 20, step_blocks=8192, min_share=1024)
    rid, alone = _submit(tx, srv, target)
    r0 = srv.wait(rid, timeout_ms=60000)
    mix = [_job(s, side_max=520) for s in range(100, 130)]
    ids = [_submit(tx, srv, j) for j in mix[:15]]
    rid2, mixed = _submit(tx, srv, target)
    ids += [_submit(tx, srv, j) for j in mix[15:]]
    r1 = srv.wait(rid2, timeout_ms=60000)
    for i, _ in ids:
        srv.wait(i, timeout_ms=60000)
    assert r0["status"] == r1["status"] == 0
    assert r1["steps"] >= r0["steps"]  # it shared steps with the others
    assert np.array_equal(alone, mixed)
    srv.close()


def test_admission_by_memory_budget(tx, cuda, oracle):
    jobs = [_job(s, side_max=200) for s in range(500, 530)]
    for j in jobs:
        j["mips"] = True
    biggest = max(j["w"] * j["h"] for j in jobs)
    budget = 3 * (biggest * 4 * 2 + (1 << 16))  # room for only a few jobs at a time
    srv = tx.Server(memory_budget=budget, step_blocks=2048, min_share=256)
    sub = [_submit(tx, srv, j) for j in jobs]
    queued = 0
    for j, (rid, out) in zip(jobs, sub):
        res = srv.wait(rid, timeout_ms=60000)
        queued += res["queue_us"] > 0
        assert np.array_equal(out, _expected(oracle, j))
    st = srv.stats()
    assert 0 < st["held_high_water"] <= budget
    assert st["memory_budget"] == budget and st["busy_us"] > 0
    # a job that can never fit is refused at once
    big = np.zeros((1024, 1024, 4), np.uint8)
    with pytest.raises(tx.TexpressoError) as e:
        srv.submit(big, 1024, 1024, tx.Format.Bc1, tx.Params(), np.zeros(tx.chain_compressed_size(0, 1024, 1024), np.uint8))
    assert e.value.status == -8
    srv.close()


def test_submit_from_many_threads(tx, cuda, oracle):
    srv = tx.Server(memory_budget=256 << 20, step_blocks=4096)
    jobs = [_job(s, side_max=120) for s in range(900, 948)]
    results = [None] * len(jobs)

    def run(lo):
        for k in range(lo, len(jobs), 4):
            rid, out = _submit(tx, srv, jobs[k])
            srv.wait(rid, timeout_ms=60000)
            results[k] = out

    ts = [threading.Thread(target=run, args=(i,)) for i in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    for j, out in zip(jobs, results):
        assert np.array_equal(out, _expected(oracle, j))
    srv.close()


def test_wait_timeout_and_cancel(tx, cuda):
    # a 26 MiB budget: the 2048x2048 job (about 24 MiB with mips) fills it,
    # the 700x700 jobs behind it wait for memory (FIFO admission)
    big = dict(img=workloads.ramp_texture(2048, 2048, seed=3), w=2048, h=2048, fmt=0, alg=2, aw=False, mips=True)
    small = [dict(img=workloads.ramp_texture(700, 700, seed=10 + s), w=700, h=700, fmt=2, alg=1, aw=False, mips=True)
             for s in range(4)]
    srv = tx.Server(memory_budget=26 << 20, step_blocks=2048, min_share=256)
    rid, _ = _submit(tx, srv, big)
    waiting = [_submit(tx, srv, j) for j in small]
    with pytest.raises(tx.TexpressoError) as e:
        srv.wait(rid, timeout_ms=0)
    assert e.value.status == -7                     # still running: timed out, job kept
    assert srv.cancel(waiting[-1][0]) is True       # queued behind the budget: dropped
    with pytest.raises(tx.TexpressoError) as e:
        srv.wait(waiting[-1][0], timeout_ms=60000)
    assert e.value.status == -11
    assert srv.wait(rid, timeout_ms=60000)["status"] == 0
    for i, _ in waiting[:-1]:
        assert srv.wait(i, timeout_ms=60000)["status"] == 0
    srv.close()


def test_admission_waits_for_free_device_memory(tx, cuda, oracle):
    """Admission follows the device's free memory, not only the budget: with
    the device filled to within the headroom (1 GiB) plus a few MiB, a job of
    about 25 MiB that the budget allows waits (the wait times out, the job is
    kept, the deferral is counted) and runs as soon as the memory is freed."""
    torch = cuda
    srv = tx.Server(memory_budget=8 << 30, step_blocks=1 << 16)
    torch.cuda.synchronize()
    free, _ = torch.cuda.mem_get_info()
    hold = free - (1 << 30) - (8 << 20)
    if hold <= 0:
        srv.close()
        pytest.skip("device has less than the headroom free")
    filler = torch.empty(hold, dtype=torch.uint8, device="cuda")
    free_now, _ = torch.cuda.mem_get_info()
    if free_now > (1 << 30) + (20 << 20):
        del filler
        srv.close()
        pytest.skip("could not fill the device to within the headroom")
    j = dict(img=workloads.ramp_texture(2048, 2048, seed=21), w=2048, h=2048, fmt=0, alg=0, aw=False, mips=True)
    rid, out = _submit(tx, srv, j)
    with pytest.raises(tx.TexpressoError) as e:
        srv.wait(rid, timeout_ms=300)
    assert e.value.status == -7
    assert srv.stats()["hbm_deferrals"] == 1
    del filler
    torch.cuda.empty_cache()
    assert srv.wait(rid, timeout_ms=60000)["status"] == 0
    assert np.array_equal(out, _expected(oracle, j))
    srv.close()
