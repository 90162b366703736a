"""The fused kernels' pair queue: launches on a handle's own compute stream take
their pairs from a device queue (CTAs on faster SMs take more), launches on a
caller's stream walk fixed pairs per CTA.  Both must give the same bits, and
the queue must be empty again after every launch, whatever the pair count:
each output buffer starts as NaN, so a launch that skipped pairs shows."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def _scene(size, side, n):
    from emida_gb300 import synth
    ref = synth.reference_pattern(size, 91)
    pics, _ = synth.deformed_patterns(size, 91, n, sigma_eps=4e-3)
    _, begins = synth.roi_grid(size, 4, side // 2, margin=side // 2 + 4)
    return ref, np.ascontiguousarray(pics), begins


@pytest.mark.parametrize("side,precision", [(64, "float"), (48, "float"), (32, "float"),
                                            (96, "float"), (128, "float"), (64, "double")])
def test_queue_and_static_walk_give_the_same_bits(side, precision):
    # side 128: the 256-point kernel on clusters of two CTAs
    import torch
    from emida_gb300 import DeviceBuffer, GpuOffset, _lib
    size = 1024 if side == 128 else 512
    ref, uniq, begins = _scene(size, side, 4)
    n_max = 200 if side == 128 else 600
    pics = np.ascontiguousarray(np.resize(uniq, (n_max, size, size)))
    d_pics = DeviceBuffer.from_array(pics)
    g = GpuOffset((size, size), begins, (side, side), (2 * side - 1, 2 * side - 1), 32, "fft", 5, 1,
                  precision, np.uint16, "fused")
    g.allocate_memory(ref)
    S = len(begins)
    other = torch.cuda.Stream()
    # pair counts below, at and far above one wave of CTAs, back to back
    for n in (1, 3, 37, n_max, 2, n_max):
        outs = []
        for stream in (None, other.cuda_stream):
            o = DeviceBuffer(n * S * 16)
            o.upload(np.full((n * S, 2), np.nan))
            g.run_device(d_pics, n, o, stream=stream)
            _lib.call("emida_gb_synchronize")
            outs.append(o.download(np.float64, (n * S, 2)))
        queued, walked = outs
        assert not np.isnan(queued).any() and not np.isnan(walked).any()
        assert np.array_equal(queued, walked)
    g.close()
