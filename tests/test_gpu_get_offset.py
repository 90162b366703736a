"""End-to-end golden vectors of the reference through the C ABI
(test/get_offset_test.cpp): FP64 input patterns, gpu_offset<double, double>."""
import json
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

EXPECTED = json.load(open(os.path.join(GOLDEN, "get_offset_expected.json")))


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def golden_pair():
    return np.load(os.path.join(GOLDEN, "data_pic.npy")), np.load(os.path.join(GOLDEN, "data_temp.npy"))


def slice_begins(src, size, step):
    return [(x, y) for y in range(0, src - size + 1, step) for x in range(0, src - size + 1, step)]


def test_get_offset_bigger():
    # test/get_offset_test.cpp:10-27 (brute, 127 x 127 lags, s = 3): 2e-14
    from emida_gb300 import get_offset
    pic, temp = golden_pair()
    offs = get_offset(pic[:64, :64], temp[:64, :64], (64, 64))
    g = EXPECTED["get_offset_single"]
    assert abs(offs[0, 0] - g["x"]) <= g["tol"]
    assert abs(offs[0, 1] - g["y"]) <= g["tol"]


@pytest.mark.parametrize("policy,mode", [("brute", "plain"), ("fft", "plain"), ("fft", "fused")])
@pytest.mark.parametrize("batch", [1, 5])
def test_get_offset_batched(policy, mode, batch):
    # test/get_offset_test.cpp:120-200: 49 ROIs x batch, 7e-13
    from emida_gb300 import GpuOffset
    pic, temp = golden_pair()
    g = EXPECTED["get_offset_batched"]
    offs_exp = np.tile(np.array(g["offsets"]), (batch, 1))
    go = GpuOffset((256, 256), slice_begins(256, 64, 32), (64, 64), (127, 127), batch, policy, 3, 1,
                   "double", np.float64, mode)
    assert go.mode == mode
    go.allocate_memory(temp)
    offs, _ = go.get_offset(np.repeat(pic[None], batch, 0))
    go.close()
    assert np.abs(offs - offs_exp).max() <= g["tol"]


@pytest.mark.parametrize("policy,mode", [("brute", "plain"), ("fft", "plain"), ("fft", "fused")])
def test_get_offset_float_within_fp32_tolerance(policy, mode):
    # FP32 compute against the FP64 golden offsets: 1e-3 px
    from emida_gb300 import GpuOffset
    pic, temp = golden_pair()
    exp = np.array(EXPECTED["get_offset_batched"]["offsets"])
    go = GpuOffset((256, 256), slice_begins(256, 64, 32), (64, 64), (127, 127), 1, policy, 3, 1,
                   "float", np.float64, mode)
    go.allocate_memory(temp)
    offs, _ = go.get_offset(pic)
    go.close()
    assert np.abs(offs - exp).max() <= 1e-3


def test_pipeline_api_matches_get_offset():
    # transfer_pic_to_device_async -> get_offset_core -> finalize
    # (src/process_files.hpp:98-233) against get_offset on the same batch
    from emida_gb300 import GpuOffset
    pic, temp = golden_pair()
    for mode in ("plain", "fused"):
        go = GpuOffset((256, 256), slice_begins(256, 64, 32), (64, 64), (127, 127), 2, "fft", 3, 2,
                       "double", np.float64, mode)
        go.allocate_memory(temp)
        batch = np.stack([pic, pic[::-1, ::-1].copy()])
        ref_offs, ref_coefs = go.get_offset(batch)
        for _ in range(3):
            buf = go.transfer_pic_to_device_async(batch)
            maxes, neigh = go.get_offset_core(buf)
            offs, coefs = go.finalize(maxes, neigh)
            assert np.array_equal(offs, ref_offs)
            assert np.array_equal(coefs, ref_coefs)
        go.close()


def test_submit_wait_pipeline_matches_get_offset():
    # several batches in flight on the three streams; partial last batch
    from emida_gb300 import EmidaError, GpuOffset
    pic, temp = golden_pair()
    begins = slice_begins(256, 64, 32)
    batches = [np.stack([pic, pic[::-1, ::-1].copy(), pic[:, ::-1].copy()]) for _ in range(4)]
    for mode in ("plain", "fused"):
        go = GpuOffset((256, 256), begins, (64, 64), (127, 127), 3, "fft", 5, 3, "float",
                       np.float64, mode)
        go.allocate_memory(temp)
        ref_offs, ref_coefs, ref_peaks = go.get_offset(batches[0], with_peaks=True)
        tickets = [go.submit(b) for b in batches[:3]]
        with pytest.raises(EmidaError, match="in flight"):
            go.submit(batches[3])
        for t in tickets:
            offs, coefs, peaks = go.wait(t, with_peaks=True)
            assert np.array_equal(offs, ref_offs) and np.array_equal(coefs, ref_coefs)
            assert np.array_equal(peaks, ref_peaks)
        with pytest.raises(EmidaError, match="unknown ticket"):
            go.wait(tickets[0])
        t = go.submit(batches[3], patterns=2)
        offs, _ = go.wait(t, patterns=2)
        assert np.array_equal(offs, ref_offs[:2 * len(begins)])
        go.close()
