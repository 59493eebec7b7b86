"""The multi-process path of bench.py on CPU: two gloo ranks, each building
its own seeded sequence with the oracle (the GPU path shards the same way,
one independent sequence per rank, no collective on the data path), joined
by the job-time reduction (maximum over ranks) and the whole-job throughput;
and two gloo ranks that each drive libwtg's C ABI in their own process
(a real build checked against the oracle where a GPU is present, the
no-GPU, argument and injected-allocation-failure paths otherwise); and a
rank that fails between steps: the other rank's next collective ends with
an error within the process group's timeout instead of hanging."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, out):
    import sys
    for p in (ROOT, os.path.join(ROOT, "wavelet-suffix-fm-index_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import datagen
    from oracle import oracle as O
    sym = datagen.exp_u32(1 << 14, seed=bench.SEED + rank)  # one sequence per rank
    bits, _ = O.wt_build(sym, bench.LEVELS)
    checksum = int(np.bitwise_xor.reduce(bits))
    seconds = 0.5 + rank  # rank 1 is the slowest
    job = bench.slowest_rank(dist, torch, seconds, torch.device("cpu"))
    value = bench.job_throughput(world, 3, 1e9, job)
    sums = torch.tensor([checksum & 0xFFFFFFFF], dtype=torch.int64)
    gathered = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(gathered, sums)
    out[rank] = (job, value, [int(g.item()) for g in gathered])
    dist.destroy_process_group()


def test_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            job, value, checks = out[r]
            assert job == pytest.approx(1.5)              # the slowest rank's time
            assert value == pytest.approx(2 * 3 * 1.0 / 1.5)  # both ranks' bytes over that time
            assert checks[0] != checks[1]                 # independent sequences


def _libwtg_rank(rank, world, port, out):
    import sys
    for p in (ROOT, os.path.join(ROOT, "wavelet-suffix-fm-index_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import datagen
    import wtg
    from oracle import oracle as O
    sym = datagen.exp_u32(1 << 15, seed=77 + rank)  # one sequence per rank
    codes = []
    try:  # argument check, before any device work
        wtg.WaveletTree(sym, levels=25)
    except wtg.WtgError as e:
        codes.append(e.code)
    checksum = 0
    try:
        wtg.inject_alloc_failure(1)
        try:
            wtg.WaveletTree(sym, levels=20)
        except wtg.WtgError as e:
            codes.append(e.code)  # ERR_OOM with a GPU, ERR_CUDA without
        wtg.inject_alloc_failure(0)
        t = wtg.WaveletTree(sym, levels=20)
        bits = t.bits()
        ref, _ = O.wt_build(sym, 20)
        codes.append(0 if np.array_equal(bits, ref) else -1)
        checksum = int(np.bitwise_xor.reduce(bits)) & 0xFFFFFFFF
        t.free()
    except wtg.WtgError as e:
        codes.append(e.code)
    finally:
        wtg.inject_alloc_failure(0)
    mine = torch.tensor(codes + [checksum], dtype=torch.int64)
    gathered = [torch.zeros_like(mine) for _ in range(world)]
    dist.all_gather(gathered, mine)
    out[rank] = [g.tolist() for g in gathered]
    dist.destroy_process_group()


def test_two_gloo_ranks_through_libwtg():
    ctx = mp.get_context("spawn")
    port = _free_port()
    has_gpu = torch.cuda.is_available()
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_libwtg_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
            assert p.exitcode == 0
        assert out[0] == out[1]  # both ranks see both ranks' results
        for codes in out[0]:
            assert codes[0] == 1  # ERR_INVALID: levels above 24
            if has_gpu:
                assert codes[1:3] == [2, 0]  # ERR_OOM injected, then an exact build
            else:
                assert codes[1:3] == [3, 3]  # ERR_CUDA: no GPU, no CPU fallback
        if has_gpu:
            assert out[0][0][-1] != out[0][1][-1]  # independent sequences


def _failing_rank(rank, world, port, out):
    import sys
    import time
    for p in (ROOT,):
        if p not in sys.path:
            sys.path.insert(0, p)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    bench.init_ranks(dist, "gloo", 5)
    bench.slowest_rank(dist, torch, 1.0, torch.device("cpu"))  # step 1: both ranks
    if rank == 1:
        raise RuntimeError("rank 1 fails between steps")
    t0 = time.perf_counter()
    try:
        bench.slowest_rank(dist, torch, 2.0, torch.device("cpu"))  # step 2: the peer is gone
        out[rank] = ("no error", time.perf_counter() - t0)
    except Exception as e:  # the collective reports the lost peer
        out[rank] = (type(e).__name__, time.perf_counter() - t0)


def test_failed_rank_ends_the_next_collective():
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_failing_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert procs[1].exitcode != 0  # the failing rank
        assert procs[0].exitcode == 0
        kind, waited = out[0]
        assert kind != "no error" and waited < 60
