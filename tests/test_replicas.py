"""The multi-GPU bench path on CPU: two gloo ranks (127.0.0.1), each with its own seed and its own
elapsed time; the job's time is the slowest rank's and the throughput counts every rank's units."""

from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from wgnet_gb300 import replicas

    r, w, local = replicas.env()
    dist = replicas.init("gloo")
    replicas.barrier(dist)
    elapsed_ms = 100.0 + 50.0 * r  # rank 1 is slower
    slowest = replicas.max_over_ranks(elapsed_ms, dist)
    rate = replicas.aggregate_rate(256, 5, w, slowest)
    out.put((r, w, local, replicas.rank_seed(0, r), slowest, rate))
    replicas.barrier(dist)
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [x[0] for x in res] == [0, 1] and all(x[1] == 2 for x in res)
    assert [x[3] for x in res] == [0, 1]          # each rank draws its own models
    assert all(x[4] == 150.0 for x in res)        # max over ranks
    assert all(x[5] == pytest.approx(2 * 256 * 5 / 0.150) for x in res)


def test_single_process_needs_no_group(monkeypatch):
    from wgnet_gb300 import replicas

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    assert replicas.env() == (0, 1, 0)
    assert replicas.init("gloo") is None
    assert replicas.max_over_ranks(12.5, None) == 12.5
