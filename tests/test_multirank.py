"""The multi-GPU bookkeeping (sharding, max-over-ranks timing, whole-job
rate) with two gloo ranks on the CPU."""
import os
import socket

import pytest

from emida_gb300.shard import max_over_ranks, pattern_shard, whole_job_rate


def test_pattern_shards_cover_once():
    for n in (0, 1, 7, 256, 1001):
        for world in (1, 2, 3, 8):
            got = []
            for r in range(world):
                a, b = pattern_shard(n, r, world)
                assert 0 <= a <= b <= n
                got.extend(range(a, b))
            assert got == list(range(n))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [3.0, 5.0][rank]
    dist.barrier()
    worst = max_over_ranks(ms, dist)
    a, b = pattern_shard(10, rank, world)
    q.put((rank, worst, whole_job_rate(25600, worst / 1000, world), (a, b)))
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_rank():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [5.0, 5.0]
    assert res[0][2] == pytest.approx(2 * 25600 / 0.005)
    assert res[0][3] == (0, 5) and res[1][3] == (5, 10)
