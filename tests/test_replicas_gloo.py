"""Multi-process host logic of the replica path (world size 2, gloo, CPU)."""
import os
import socket

import pytest

from pynufft_gb300.replicas import shard


def test_shard_covers_units_exactly():
    for n in (0, 1, 7, 64, 65):
        for world in (1, 2, 3, 8):
            parts = [shard(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            for (a, b), (c, d) in zip(parts, parts[1:]):
                assert b == c
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    from pynufft_gb300.replicas import job_rate, max_over_ranks, shard, sum_over_ranks
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        start, stop = shard(64, rank, world)
        t = 1.0 + rank                       # rank 1 is the slow one
        q.put((rank, max_over_ranks(t), sum_over_ranks(stop - start), job_rate(stop - start, t)))
    finally:
        dist.destroy_process_group()


def test_two_rank_max_time_and_job_rate():
    import multiprocessing as mp
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=120) for _ in ps]
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, tmax, total, rate in res:
        assert tmax == 2.0
        assert total == 64
        assert rate == pytest.approx(32.0)
