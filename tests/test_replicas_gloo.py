"""The multi-process path of bench.py on CPU: two gloo ranks, each building
its own seeded sequence with the oracle (the GPU path shards the same way,
one independent sequence per rank, no collective on the data path), joined
by the job-time reduction (maximum over ranks) and the whole-job throughput."""
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
