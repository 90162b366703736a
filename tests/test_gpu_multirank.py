"""Two ranks through the library, the way bench.py runs N GPUs: each rank
selects its device in the library (emida_gb_set_device), takes its contiguous
shard of the patterns and runs it with no collective on the data path; the
ranks meet over gloo only to gather their results and the slowest rank's
time.  On one GPU both ranks use device 0: their kernels never wait on each
other.  The gathered offsets must equal one process's run of all patterns bit
for bit, and the peaks the FP64 oracle's."""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIZE, P, SIDE, FIT = 256, 6, 32, 5


def scene():
    from emida_gb300 import synth
    ref = synth.reference_pattern(SIZE, 41)
    pics, _ = synth.deformed_patterns(SIZE, 41, P, sigma_eps=5e-3)
    _, begins = synth.roi_grid(SIZE, 3, SIDE // 2, margin=40)
    return ref, np.ascontiguousarray(pics), np.asarray(begins, dtype=np.uint32)


def run(ref, pics, begins):
    from emida_gb300 import GpuOffset
    g = GpuOffset((SIZE, SIZE), begins, (SIDE, SIDE), None, len(pics), "fft", FIT, 1, "float",
                  np.uint16, "fused")
    g.allocate_memory(ref)
    offs, coefs, peaks = g.get_offset(pics, with_peaks=True)
    g.close()
    return offs, peaks


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import time

    import torch.distributed as dist
    from emida_gb300 import _lib, device_count
    from emida_gb300.shard import max_over_ranks, pattern_shard
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    _lib.call("emida_gb_set_device", rank % device_count())
    ref, pics, begins = scene()
    a, b = pattern_shard(P, rank, world)
    dist.barrier()
    t0 = time.perf_counter()
    offs, peaks = run(ref, pics[a:b], begins)
    ms = 1000 * (time.perf_counter() - t0)
    worst = max_over_ranks(ms, dist)
    parts = [None] * world
    dist.all_gather_object(parts, (a, b, offs, peaks))
    if rank == 0:
        q.put((worst, parts))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_patterns_and_match_one_process():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    import __graft_entry__
    __graft_entry__.build_library()
    from oracle import oracle as eo
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    worst, parts = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert worst > 0
    parts.sort(key=lambda x: x[0])
    assert [(a, b) for a, b, _, _ in parts] == [(0, 3), (3, 6)]
    offs = np.concatenate([o for _, _, o, _ in parts])
    peaks = np.concatenate([k for _, _, _, k in parts])
    ref, pics, begins = scene()
    one_offs, one_peaks = run(ref, pics, begins)
    assert np.array_equal(offs, one_offs)
    assert np.array_equal(peaks, one_peaks)
    _, _, o_peaks = eo.get_offsets(ref, pics, begins, SIDE, SIDE, eo.POLICY_FFT, FIT)
    assert np.array_equal(peaks, o_peaks)
