"""Edge cases through the C ABI against the FP64 oracle: ROIs that touch every
border of the pattern (x not a multiple of 8 as well, so the fused kernels'
16-byte-aligned TMA box reaches past the right edge and reads the fill), flat
patterns whose maps are all ties (the first maximum wins everywhere), and empty
requests (no patterns)."""
import numpy as np
import pytest

from tests.test_gpu_synthetic import assert_offsets, oracle, run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def border_rois(size, side):
    e = size - side
    return np.array([[0, 0], [e, 0], [0, e], [e, e], [5, e // 2], [e - 3, 7], [e // 2 + 1, e]],
                    dtype=np.uint32)


@pytest.fixture(scope="module")
def scene160():
    from emida_gb300 import synth
    ref = synth.reference_pattern(160, 77)
    pics, _ = synth.deformed_patterns(160, 77, 3, sigma_eps=3e-3)
    return ref, np.ascontiguousarray(pics)


@pytest.mark.parametrize("precision,mode,tol", [("float", "fused", 1e-3), ("double", "fused", 1e-9),
                                                ("float", "plain", 1e-3), ("double", "plain", 1e-9)])
def test_fft_rois_on_every_border(scene160, precision, mode, tol):
    ref, pics = scene160
    begins = border_rois(160, 32)
    offs, coefs, peaks = run(ref, pics, begins, 32, "fft", 5, precision, mode)
    o_offs, o_coefs, o_peaks = oracle(ref, pics, begins, 32, "fft", 5)
    assert np.array_equal(peaks, o_peaks)
    assert_offsets(offs, coefs, o_offs, o_coefs, 5, tol)


def test_brute_rois_on_every_border_bit_exact(scene160):
    ref, pics = scene160
    begins = border_rois(160, 32)
    offs, coefs, peaks = run(ref, pics, begins, 32, "brute", 3, "double", "plain")
    o_offs, o_coefs, o_peaks = oracle(ref, pics, begins, 32, "brute", 3)
    assert np.array_equal(peaks, o_peaks)
    assert np.array_equal(offs, o_offs) and np.array_equal(coefs, o_coefs)


def test_tensor_rois_on_every_border():
    from emida_gb300 import synth
    ref = synth.reference_pattern(192, 78)
    pics, _ = synth.deformed_patterns(192, 78, 2, sigma_eps=3e-3)
    begins = border_rois(192, 64)
    offs, coefs, peaks = run(ref, pics, begins, 64, "brute", 5, "float", "tensor")
    o_offs, o_coefs, o_peaks = oracle(ref, pics, begins, 64, "brute", 5)
    assert np.array_equal(peaks, o_peaks)
    assert_offsets(offs, coefs, o_offs, o_coefs, 5, 1e-2)


@pytest.mark.parametrize("policy,precision,mode", [("fft", "float", "fused"), ("fft", "double", "fused"),
                                                   ("fft", "float", "plain"), ("brute", "double", "plain"),
                                                   ("brute", "float", "tensor")])
def test_flat_patterns_tie_everywhere(policy, precision, mode):
    """Constant patterns: every prepared ROI is zero, so is every map value, and
    the peak is the map's first index, as in the oracle.  The fit of an all-zero
    neighbourhood has no extremum; its offsets must match the oracle's bits,
    NaN for NaN."""
    side = 64 if mode == "tensor" else 32
    size = 192
    ref = np.full((size, size), 1000, dtype=np.uint16)
    pics = np.full((2, size, size), 1234, dtype=np.uint16)
    begins = np.array([[0, 0], [64, 40], [size - side, size - side]], dtype=np.uint32)
    offs, coefs, peaks = run(ref, pics, begins, side, policy, 3, precision, mode)
    o_offs, o_coefs, o_peaks = oracle(ref, pics, begins, side, policy, 3)
    assert np.array_equal(peaks, o_peaks)
    assert np.array_equal(coefs, o_coefs)
    assert np.array_equal(offs, o_offs, equal_nan=True)


def test_empty_requests():
    from emida_gb300 import DeviceBuffer, EmidaError, GpuOffset, MultiLayout, Server, synth
    ref = synth.reference_pattern(128, 79)
    begins = np.array([[16, 16], [64, 48]], dtype=np.uint32)
    g = GpuOffset((128, 128), begins, (32, 32), None, 4, "fft", 3, 2, "float", np.uint16, "fused")
    g.allocate_memory(ref)
    d_pics = DeviceBuffer(4 * 128 * 128 * 2)
    d_offs = DeviceBuffer(4 * 2 * 16)
    d_offs.upload(np.full((8, 2), 7.0))
    # no patterns on the device: nothing runs, nothing is written
    g.run_device(d_pics, 0, d_offs)
    from emida_gb300 import _lib
    _lib.call("emida_gb_synchronize")
    assert np.array_equal(d_offs.download(np.float64, (8, 2)), np.full((8, 2), 7.0))
    # an empty batch is refused before any device work
    with pytest.raises(EmidaError):
        g.submit(np.zeros((1, 128, 128), np.uint16), patterns=0)
    g.close()
    # the multi-layout planner with no patterns
    m = MultiLayout((128, 128), "float")
    m.add_layout(begins, 32, 3, ref)
    m.run(d_pics, np.zeros(0, np.uint32), d_offs, graph=False)
    m.synchronize()
    assert np.array_equal(d_offs.download(np.float64, (8, 2)), np.full((8, 2), 7.0))
    m.close()
    # the request loop refuses a row of no patterns
    srv = Server("float", hbm_bytes=64 << 20, step_patterns=8)
    lid = srv.add_layout((128, 128), begins, 32, 3, ref)
    with pytest.raises(EmidaError):
        srv.submit(lid, np.zeros((0, 128, 128), np.uint16))
    srv.close()
