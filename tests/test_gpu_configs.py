"""Parity at the benchmark workloads' own shapes, against the FP64 oracle.

- Plain brute form, FP64, s=3: 16 deformed 512^2 patterns (eps ~ N(0, 2e-3)),
  25 ROIs of 64^2 on a 5x5 grid, the 127x127 lag window.  Bit-exact.
- Detector form: 40 deformed 1024^2 patterns (eps ~ N(0, 5e-3)), 100 ROIs of
  64^2 on a 10x10 grid, FFT (128^2 transforms), s=5, batch size 32, so the
  submit/wait stream ends in a short batch of 8.  Float within 1e-3 px,
  double within 1e-9 px, fused and plain, through get_offset and submit/wait.
- Precision form: the tensor-core brute contraction at s=7 on 1024^2 patterns
  with 100 ROIs, within 1e-2 px.
- Batching form: a radius-64 layout (the 256-point cluster kernel) at fit size
  9, alone and with radii 16/24/32/48 in one multi-layout run under a captured
  graph.

In every case the integer peaks equal the oracle's.  The oracle runs on a
thread pool over patterns (its C calls release the GIL)."""
import concurrent.futures as cf
import os

import numpy as np
import pytest

from tests.test_gpu_synthetic import assert_offsets, well_posed

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def oracle_parallel(ref, pics, begins, side, policy, s, cross=None):
    """eo.get_offsets pattern by pattern on all host cores, concatenated."""
    from oracle import oracle as eo
    pol = eo.POLICY_FFT if policy == "fft" else eo.POLICY_BRUTE
    cw, ch = cross or (2 * side - 1, 2 * side - 1)

    def one(p):
        return eo.get_offsets(ref, pics[p:p + 1], begins, side, side, pol, s, cw, ch)

    eo.lib()  # load (and build if needed) before the threads start
    with cf.ThreadPoolExecutor(max_workers=min(len(pics), os.cpu_count() or 1)) as ex:
        parts = list(ex.map(one, range(len(pics))))
    return tuple(np.concatenate([p[k] for p in parts]) for k in range(3))


def handle(ref, begins, side, cross, batch, policy, s, precision, mode, src, in_buffers=1):
    from emida_gb300 import GpuOffset
    g = GpuOffset((src, src), begins, (side, side), cross, batch, policy, s, in_buffers, precision,
                  np.uint16, mode)
    g.allocate_memory(ref)
    assert g.mode == mode
    return g


def submit_all(g, host, batch):
    """Every pattern of `host` through submit/wait in batches of `batch` (the
    last one short), two batches in flight."""
    n = len(host)
    starts = list(range(0, n, batch))
    offs, coefs, peaks = [None] * len(starts), [None] * len(starts), [None] * len(starts)
    pending = []
    for i, k in enumerate(starts):
        pending.append((i, g.submit(host[k:k + batch])))
        if len(pending) == 2:
            j, t = pending.pop(0)
            offs[j], coefs[j], peaks[j] = g.wait(t, with_peaks=True)
    for j, t in pending:
        offs[j], coefs[j], peaks[j] = g.wait(t, with_peaks=True)
    return np.concatenate(offs), np.concatenate(coefs), np.concatenate(peaks)


# ---- plain brute form, FP64: 16 x 512^2, 5 x 5 ROIs, s = 3 ---------------------------

@pytest.fixture(scope="module")
def brute512():
    from emida_gb300 import synth
    ref = synth.reference_pattern(512, seed=3)
    pics, _ = synth.deformed_patterns(512, 3, 16, sigma_eps=2e-3)
    _, begins = synth.roi_grid(512, 5, 32, margin=40)
    return ref, pics, begins, oracle_parallel(ref, pics, begins, 64, "brute", 3, (127, 127))


def test_plain_brute_fp64_16x512_bit_exact(brute512):
    from emida_gb300 import pinned_array
    ref, pics, begins, (o_offs, o_coefs, o_peaks) = brute512
    g = handle(ref, begins, 64, (127, 127), 16, "brute", 3, "double", "plain", 512, in_buffers=2)
    offs, coefs, peaks = g.get_offset(pics, with_peaks=True)
    assert len(offs) == 16 * 25
    assert np.array_equal(peaks, o_peaks)
    assert np.array_equal(offs, o_offs)
    assert np.array_equal(coefs, o_coefs)
    host = pinned_array(pics.shape)
    host[:] = pics
    s_offs, s_coefs, s_peaks = submit_all(g, host, 16)
    g.close()
    assert np.array_equal(s_peaks, o_peaks)
    assert np.array_equal(s_offs, o_offs) and np.array_equal(s_coefs, o_coefs)


# ---- detector form: 40 x 1024^2, 10 x 10 ROIs of r = 32, FFT, s = 5, batch 32 -----------

@pytest.fixture(scope="module")
def detector():
    from emida_gb300 import pinned_array, synth
    ref = synth.reference_pattern(1024, seed=2024)
    pics, _ = synth.deformed_patterns(1024, 2024, 40, sigma_eps=5e-3)
    _, begins = synth.roi_grid(1024, 10, 32, margin=40)
    host = pinned_array(pics.shape)
    host[:] = pics
    return ref, pics, host, begins, oracle_parallel(ref, pics, begins, 64, "fft", 5)


@pytest.mark.parametrize("mode", ["fused", "plain"])
@pytest.mark.parametrize("precision,tol", [("float", 1e-3), ("double", 1e-9)])
def test_detector_40x1024_fft(detector, mode, precision, tol):
    ref, pics, host, begins, (o_offs, o_coefs, o_peaks) = detector
    g = handle(ref, begins, 64, (127, 127), 32, "fft", 5, precision, mode, 1024, in_buffers=3)
    # get_offset on the first whole batch
    offs, coefs, peaks = g.get_offset(pics[:32], with_peaks=True)
    n32 = 32 * 100
    assert np.array_equal(peaks, o_peaks[:n32])
    assert_offsets(offs, coefs, o_offs[:n32], o_coefs[:n32], 5, tol)
    # all 40 through submit/wait: batches of 32 and 8 from pinned memory
    s_offs, s_coefs, s_peaks = submit_all(g, host, 32)
    g.close()
    assert len(s_offs) == 40 * 100
    assert np.array_equal(s_peaks, o_peaks)
    assert_offsets(s_offs, s_coefs, o_offs, o_coefs, 5, tol)
    # the same batch gives the same bits whichever entry point ran it
    assert np.array_equal(s_offs[:n32], offs) and np.array_equal(s_coefs[:n32], coefs)


# ---- precision form: tensor-core brute at s = 7 on 1024^2, 100 ROIs --------------------

def test_tensor_s7_1024_within_1e2(detector):
    ref, pics, host, begins, _ = detector
    sel = pics[:8]
    o_offs, o_coefs, o_peaks = oracle_parallel(ref, sel, begins, 64, "brute", 7, (127, 127))
    g = handle(ref, begins, 64, (127, 127), 8, "brute", 7, "float", "tensor", 1024)
    offs, coefs, peaks = g.get_offset(sel, with_peaks=True)
    g.close()
    assert np.array_equal(peaks, o_peaks)
    ok = well_posed(o_coefs, 7)
    assert ok.mean() > 0.5
    assert np.abs(offs - o_offs)[ok].max() <= 1e-2
    scale = np.abs(o_coefs).max(axis=1, keepdims=True)
    assert (np.abs(coefs - o_coefs) <= 1e-3 * scale).all()


# ---- batching form: radius 64 (256-point cluster kernel) at fit size 9 ----------------

@pytest.fixture(scope="module")
def batching():
    from emida_gb300 import synth
    ref = synth.reference_pattern(1024, seed=77)
    pics, _ = synth.deformed_patterns(1024, 77, 6, sigma_eps=5e-3)
    layouts = []
    for i, (r, s, n) in enumerate([(64, 9, 24), (16, 3, 60), (24, 5, 40), (32, 7, 30), (48, 9, 20)]):
        _, b = synth.random_layout(1024, 700 + i, r, n, margin=4)
        layouts.append((b, 2 * r, s))
    return ref, pics, layouts


def test_radius64_fit9_fused_cluster(batching):
    ref, pics, layouts = batching
    begins, side, s = layouts[0]
    o_offs, o_coefs, o_peaks = oracle_parallel(ref, pics[:4], begins, side, "fft", s)
    g = handle(ref, begins, side, (2 * side - 1, 2 * side - 1), 4, "fft", s, "float", "fused", 1024)
    offs, coefs, peaks = g.get_offset(pics[:4], with_peaks=True)
    g.close()
    assert np.array_equal(peaks, o_peaks)
    assert_offsets(offs, coefs, o_offs, o_coefs, s, 1e-3)


def test_uneven_layouts_one_graph_run(batching):
    from emida_gb300 import DeviceBuffer, MultiLayout
    ref, pics, layouts = batching
    m = MultiLayout((1024, 1024), "float")
    for b, side, s in layouts:
        m.add_layout(b, side, s, ref)
    layout_of = np.array([0, 1, 2, 3, 4, 0], dtype=np.uint32)
    total = m.count(layout_of)
    d_pics = DeviceBuffer.from_array(pics)
    d_offs, d_coefs = DeviceBuffer(total * 16), DeviceBuffer(total * 48)
    d_max = DeviceBuffer(total * m.data_index.itemsize)
    m.run(d_pics, layout_of, d_offs, d_coefs, d_max, graph=True)
    m.synchronize()
    offs = d_offs.download(np.float64, (total, 2))
    coefs = d_coefs.download(np.float64, (total, 6))
    peaks = d_max.download(m.data_index, total)["index"]
    m.close()
    start = 0
    for p, lid in enumerate(layout_of):
        b, side, s = layouts[lid]
        n = len(b)
        o_offs, o_coefs, o_peaks = oracle_parallel(ref, pics[p:p + 1], b, side, "fft", s)
        sl = slice(start, start + n)
        assert np.array_equal(peaks[sl], o_peaks), (p, side)
        assert_offsets(offs[sl], coefs[sl], o_offs, o_coefs, s, 1e-3)
        start += n
    assert start == total
