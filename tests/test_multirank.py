"""The multi-GPU host side with two gloo ranks on the CPU: sharding,
max-over-ranks timing, the whole-job rate, and each rank loading the library
and gathering its shard's results."""
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


def _oracle_rank(rank, world, port, q):
    import numpy as np
    import torch.distributed as dist
    from emida_gb300 import _lib, device_count, synth
    from oracle import oracle as eo
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # the library loads in every rank; without a GPU its device selection
    # fails with a status, not a crash
    status = _lib.lib().emida_gb_set_device(rank)
    ref = synth.reference_pattern(128, 5)
    pics, _ = synth.deformed_patterns(128, 5, 5, sigma_eps=5e-3)
    _, begins = synth.roi_grid(128, 2, 8, margin=20)
    a, b = pattern_shard(len(pics), rank, world)
    offs, _, peaks = eo.get_offsets(ref, pics[a:b], begins, 16, 16, eo.POLICY_FFT, 3)
    parts = [None] * world
    dist.all_gather_object(parts, (a, b, offs, peaks))
    if rank == 0:
        q.put((device_count(), status, parts))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_load_the_library_and_gather_their_shards():
    """The rank flow of bench.py on the CPU: each rank loads the library and
    asks for its device, takes its shard and gathers; the oracle stands in
    for the GPU path (the GPU-marked multirank test runs the library itself)."""
    pytest.importorskip("torch")
    import numpy as np
    import torch.multiprocessing as mp

    import __graft_entry__
    __graft_entry__.build_library()
    from emida_gb300 import device_count, synth
    from oracle import oracle as eo
    if device_count() > 0:
        pytest.skip("a GPU is present: tests/test_gpu_multirank.py covers the ranks")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_oracle_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    count, status, parts = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert count == 0 and status != 0
    parts.sort(key=lambda x: x[0])
    assert [(a, b) for a, b, _, _ in parts] == [(0, 3), (3, 5)]
    ref = synth.reference_pattern(128, 5)
    pics, _ = synth.deformed_patterns(128, 5, 5, sigma_eps=5e-3)
    _, begins = synth.roi_grid(128, 2, 8, margin=20)
    offs, _, peaks = eo.get_offsets(ref, pics, begins, 16, 16, eo.POLICY_FFT, 3)
    assert np.array_equal(np.concatenate([o for _, _, o, _ in parts]), offs)
    assert np.array_equal(np.concatenate([k for _, _, _, k in parts]), peaks)
