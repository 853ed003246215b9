"""Replica timing of `bench.py --gpus N` on CPU: two gloo ranks.

The path does not shard (one grid per GPU, replicas only), so the only
multi-rank logic is the timing: every rank times its own steps, the job takes
the slowest rank's time (one all_reduce MAX), and the rate counts every
replica's particles.  These run as two spawned processes over gloo on
127.0.0.1, with no GPU.
"""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        ms_mine = 10.0 + 7.5 * rank                         # rank 1 is the slow one
        ms = bench.max_over_ranks(ms_mine, w, 'cpu')
        rate = bench.whole_job_rate(1000, 4, w, ms)
        dist.barrier()
        out.put((r, w, local, ms, rate))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context('spawn')
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [r[:3] for r in res] == [(0, 2, 0), (1, 2, 1)]
    for _, _, _, ms, rate in res:
        assert ms == 17.5                                   # every rank sees the max
        assert rate == pytest.approx(1000 * 4 * 2 / 17.5e-3)


def test_one_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.25, 1, 'cpu') == 12.25
    assert bench.whole_job_rate(1 << 30, 10, 1, 46.25) == pytest.approx((1 << 30) * 10 / 46.25e-3)
