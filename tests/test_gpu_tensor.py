"""The tensor-core brute form (tcgen05, BF16 hi/lo split operands, FP32
accumulation) against the FP64 oracle and against the staged FP32 brute path
(src/cross_corr.cu:11-74 and the stages after it).  The split keeps about 16
significant bits per product, so offsets are held to 1e-2 px and map values to
a relative 1e-4 of the peak; the integer peak must be the oracle's."""
import numpy as np
import pytest

from tests.test_gpu_synthetic import oracle, well_posed

pytestmark = pytest.mark.gpu

TOL_PX = 1e-2      # BF16-split offset tolerance
TOL_MAP = 1e-4     # map values, relative to the pair's peak


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


@pytest.fixture(scope="module")
def data512():
    from emida_gb300 import synth
    ref = synth.reference_pattern(512, seed=21)
    pics, _ = synth.deformed_patterns(512, 21, 8, sigma_eps=2e-3)
    return ref, pics


def handle(ref, begins, batch, s, mode, precision="float", src=512):
    from emida_gb300 import GpuOffset
    g = GpuOffset((src, src), begins, (64, 64), (127, 127), batch, "brute", s, 1, precision,
                  np.uint16, mode)
    g.allocate_memory(ref)
    assert g.mode == mode
    return g


@pytest.mark.parametrize("s", [3, 5, 7, 9])
def test_tensor_against_oracle(data512, s):
    from emida_gb300 import synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 5, 32, margin=40)
    g = handle(ref, begins, 3, s, "tensor")
    offs, coefs, peaks = g.get_offset(pics[:3], with_peaks=True)
    g.close()
    o_offs, o_coefs, o_peaks = oracle(ref, pics[:3], begins, 64, "brute", s)
    assert np.array_equal(peaks, o_peaks)
    ok = well_posed(o_coefs, s)
    assert ok.mean() > 0.5
    assert np.abs(offs - o_offs)[ok].max() <= TOL_PX
    scale = np.abs(o_coefs).max(axis=1, keepdims=True)
    assert (np.abs(coefs - o_coefs) <= 1e-3 * scale).all()


def test_tensor_many_pairs_per_cta(data512):
    """1000 pairs over one CTA per SM: each CTA walks several pairs and
    crosses ROI boundaries, so the reference operand is rewritten mid-run."""
    from emida_gb300 import synth
    ref, pics = data512
    batch = 40
    batch_pics = np.ascontiguousarray(np.resize(pics, (batch, 512, 512)))
    _, begins = synth.roi_grid(512, 5, 32, margin=40)
    t = handle(ref, begins, batch, 5, "tensor")
    p = handle(ref, begins, batch, 5, "plain")
    offs, coefs, peaks = t.get_offset(batch_pics, with_peaks=True)
    p_offs, p_coefs, p_peaks = p.get_offset(batch_pics, with_peaks=True)
    t.close()
    p.close()
    assert np.array_equal(peaks, p_peaks)
    ok = well_posed(p_coefs, 5)
    assert np.abs(offs - p_offs)[ok].max() <= TOL_PX
    # identical patterns repeat every 8: their results are identical too
    o = offs.reshape(batch, -1, 2)
    assert np.array_equal(o[0], o[8]) and np.array_equal(o[3], o[35])


def test_tensor_maxes_and_neighbours(data512):
    """get_offset_core's outputs (data_index<float> maxes, s x s neighbours)
    against the staged FP32 brute path."""
    from emida_gb300 import synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 4, 32, margin=48)
    out = {}
    for mode in ("tensor", "plain"):
        g = handle(ref, begins, 2, 7, mode)
        g.transfer_pic_to_device_async(pics[:2])
        maxes, neigh = g.get_offset_core(0)
        offs, coefs = g.finalize(maxes, neigh)
        out[mode] = (maxes.copy(), neigh.copy(), offs)
        g.close()
    (tm, tn, to), (pm, pn, po) = out["tensor"], out["plain"]
    assert np.array_equal(tm["index"], pm["index"])
    peak = np.abs(pm["data"]).astype(np.float64)
    assert (np.abs(tm["data"] - pm["data"]) <= TOL_MAP * peak).all()
    nb = tn.reshape(len(peak), -1).astype(np.float64) - pn.reshape(len(peak), -1)
    assert (np.abs(nb) <= TOL_MAP * peak[:, None]).all()


# (pattern +blob, reference +blob) positions inside the 64 x 64 ROI; each
# ROI also holds a -blob one pixel further along, so every ROI's pixels sum to
# 64*64 times the background and the prepared background is exactly zero.  The
# only positive lag is then (p - r) + 63: next to the lag window's edges.
EDGE_CASES = [((62, 1), (1, 62), (-1, 0)),   # lag (124, 2): top-right
              ((1, 30), (62, 30), (1, 0)),   # lag (2, 63): left
              ((30, 1), (30, 62), (0, 1)),   # lag (63, 2): top
              ((1, 1), (62, 62), (1, 1)),    # lag (2, 2): top-left
              ((20, 62), (20, 1), (0, -1)),  # lag (63, 124): bottom
              ((62, 62), (1, 1), (-1, -1))]  # lag (124, 124): bottom-right


@pytest.mark.parametrize("s", [3, 9])
def test_tensor_peaks_at_the_window_edges(s):
    src = 256
    ref = np.full((src, src), 20000, np.uint16)
    pic = ref.copy()
    begins = np.array([(64 * (k % 4), 64 * (k // 4)) for k in range(len(EDGE_CASES))], np.uint32)
    for (bx, by), ((px, py), (rx, ry), (vx, vy)) in zip(begins.tolist(), EDGE_CASES):
        pic[by + py, bx + px] += 10000
        pic[by + py + vy, bx + px + vx] -= 10000
        ref[by + ry, bx + rx] += 10000
        ref[by + ry + vy, bx + rx + vx] -= 10000
    t = handle(ref, begins, 1, s, "tensor", src=src)
    offs, coefs, peaks = t.get_offset(pic[None], with_peaks=True)
    t.close()
    o_offs, o_coefs, o_peaks = oracle(ref, pic[None], begins, 64, "brute", s)
    expect = [(p[0] - r[0] + 63) + 127 * (p[1] - r[1] + 63) for p, r, _ in EDGE_CASES]
    assert np.array_equal(o_peaks, expect)
    assert np.array_equal(peaks, o_peaks)
    # the reference reads a window that runs past the bottom of the map from
    # the next map in its batch; this form reads zeros there, so those cases
    # are compared only where the window stays inside the map
    r = (s - 1) // 2
    inside = np.array([(p[1] - q[1] + 63) + r <= 126 for p, q, _ in EDGE_CASES])
    scale = np.abs(o_coefs).max(axis=1, keepdims=True)
    assert (np.abs(coefs - o_coefs) <= 1e-3 * scale)[inside].all()
    assert inside.sum() >= 4


def test_tensor_run_device_twice_same_result(data512):
    """Back-to-back device runs through the persistent kernel give the same bits."""
    from emida_gb300 import DeviceBuffer, _lib, synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 5, 32, margin=40)
    g = handle(ref, begins, 8, 5, "tensor")
    d = DeviceBuffer.from_array(np.ascontiguousarray(pics))
    o1, o2 = DeviceBuffer(8 * 25 * 16), DeviceBuffer(8 * 25 * 16)
    g.run_device(d, 8, o1)
    g.run_device(d, 8, o2)
    _lib.call("emida_gb_synchronize")
    a, b = o1.download(np.float64, (200, 2)), o2.download(np.float64, (200, 2))
    g.close()
    assert np.array_equal(a, b)
