"""Replica logic across ranks (pbte_gb300.replicas), on CPU with gloo and
world size 2: the max-over-ranks of the elapsed time, the whole-job
throughput, and the rank environment -- what bench.py uses for N > 1."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pbte_gb300.replicas import max_over_ranks, rank_info, replica_throughput


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        info = rank_info()
        seconds = 1.5 + rank          # rank 1 is the slow one
        slowest = max_over_ranks(seconds, dist)
        dist.barrier()
        out.put((info.rank, info.world, slowest, replica_throughput(6, slowest, info.world)))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_throughput_gloo_world2():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    for rank, (r, w, slowest, thr) in enumerate(res):
        assert (r, w) == (rank, world)
        assert slowest == pytest.approx(2.5)          # the slower rank's time on every rank
        assert thr == pytest.approx(2 * 6 / 2.5)      # N * solves / max seconds


def test_single_process_defaults():
    info = rank_info({})
    assert (info.world, info.rank, info.local) == (1, 0, 0) and info.is_root
    assert max_over_ranks(3.0, None) == 3.0
    assert replica_throughput(6, 2.0, 1) == pytest.approx(3.0)
    with pytest.raises(ValueError):
        replica_throughput(6, 0.0, 1)
