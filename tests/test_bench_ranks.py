"""bench.py's multi-rank glue on CPU with the gloo backend (world size 2):
every rank embeds its own replica, the step time reported is the maximum
over ranks, and only rank 0 runs the CPU reference arm."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(None)
        got = bench.max_over_ranks(1.5 + rank, None)
        w, r, lr = bench.dist_env()
        q.put((rank, got, w, r, lr))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    results = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in results] == [2.5, 2.5]
    assert [(r[2], r[3], r[4]) for r in results] == [(2, 0, 0), (2, 1, 1)]


def test_reference_arm_non_zero_rank_exits(monkeypatch):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        steps, warmup, gpus = 1, 0, 2

    assert bench.run_reference(Args()) == 0  # no work on ranks other than 0
