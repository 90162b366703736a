"""The reference's own staged GPU pipeline (its gpu_offset<T, uint16_t> with
cuFFT, compiled from its sources by oracle/Makefile target `ref_gpu`) on the
same inputs as this library:

- its FP64 results pin the oracle a second time (peaks identical, offsets
  within 1e-9 px where the fit is well posed);
- this library's fused FP32 and FP64 forms and its tensor form agree with the
  reference's own --precision double results: identical integer peaks,
  offsets within 1e-3 px (FP32), 1e-9 px (FP64) and 1e-2 px (BF16 split).

Skipped where the reference's sources were not staged into baseline/_ref."""
import numpy as np
import pytest

from tests.test_gpu_synthetic import assert_offsets, well_posed

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()
    from oracle import ref_gpu
    if not ref_gpu.available():
        pytest.skip("the reference's sources are not staged into baseline/_ref")


@pytest.fixture(scope="module")
def scene():
    from emida_gb300 import pinned_array, synth
    ref = synth.reference_pattern(1024, seed=31)
    pics, _ = synth.deformed_patterns(1024, 31, 8, sigma_eps=5e-3)
    _, begins = synth.roi_grid(1024, 10, 32, margin=40)
    host = pinned_array(pics.shape)
    host[:] = pics
    return ref, pics, host, begins


def reference_run(ref, host, begins, policy, s, precision, cross=None):
    from oracle.ref_gpu import RefGpuOffset
    g = RefGpuOffset(ref, begins, 64, len(host), policy, s, precision, cross)
    try:
        return g.run_batch(host)
    finally:
        g.close()


def test_reference_fp64_fft_pins_the_oracle(scene):
    from tests.test_gpu_configs import oracle_parallel
    ref, pics, host, begins = scene
    r_offs, r_coefs, r_peaks = reference_run(ref, host, begins, "fft", 5, "double")
    o_offs, o_coefs, o_peaks = oracle_parallel(ref, pics, begins, 64, "fft", 5)
    assert np.array_equal(r_peaks, o_peaks)
    assert_offsets(r_offs, r_coefs, o_offs, o_coefs, 5, 1e-9)


def test_reference_fp64_brute_pins_the_oracle(scene):
    from tests.test_gpu_configs import oracle_parallel
    ref, pics, host, begins = scene
    sel = np.ascontiguousarray(host[:2])
    from emida_gb300 import pinned_array
    pin = pinned_array(sel.shape)
    pin[:] = sel
    r_offs, r_coefs, r_peaks = reference_run(ref, pin, begins, "brute", 3, "double", 127)
    o_offs, o_coefs, o_peaks = oracle_parallel(ref, pics[:2], begins, 64, "brute", 3, (127, 127))
    assert np.array_equal(r_peaks, o_peaks)
    assert_offsets(r_offs, r_coefs, o_offs, o_coefs, 3, 1e-9)


@pytest.mark.parametrize("mode,precision,tol", [("fused", "float", 1e-3), ("fused", "double", 1e-9),
                                                ("plain", "float", 1e-3)])
def test_library_agrees_with_the_references_fp64_run(scene, mode, precision, tol):
    from emida_gb300 import GpuOffset
    ref, pics, host, begins = scene
    r_offs, r_coefs, r_peaks = reference_run(ref, host, begins, "fft", 5, "double")
    g = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), len(pics), "fft", 5, 1, precision,
                  np.uint16, mode)
    g.allocate_memory(ref)
    offs, coefs, peaks = g.get_offset(pics, with_peaks=True)
    g.close()
    assert np.array_equal(peaks, r_peaks)
    assert_offsets(offs, coefs, r_offs, r_coefs, 5, tol)


def test_tensor_form_agrees_with_the_references_fp64_brute_run(scene):
    from emida_gb300 import GpuOffset, pinned_array
    ref, pics, host, begins = scene
    pin = pinned_array((2,) + pics.shape[1:])
    pin[:] = pics[:2]
    r_offs, r_coefs, r_peaks = reference_run(ref, pin, begins, "brute", 7, "double", 127)
    g = GpuOffset((1024, 1024), begins, (64, 64), (127, 127), 2, "brute", 7, 1, "float", np.uint16,
                  "tensor")
    g.allocate_memory(ref)
    offs, coefs, peaks = g.get_offset(pics[:2], with_peaks=True)
    g.close()
    assert np.array_equal(peaks, r_peaks)
    ok = well_posed(r_coefs, 7)
    assert ok.mean() > 0.5
    assert np.abs(offs - r_offs)[ok].max() <= 1e-2


def test_reference_fp32_fft_is_within_its_own_tolerance(scene):
    """The reference's FP32 run against its FP64 run: the FP32 tolerance of
    1e-3 px holds for the reference itself on this input."""
    ref, pics, host, begins = scene
    d_offs, d_coefs, d_peaks = reference_run(ref, host, begins, "fft", 5, "double")
    f_offs, f_coefs, f_peaks = reference_run(ref, host, begins, "fft", 5, "float")
    assert np.array_equal(f_peaks, d_peaks)
    ok = well_posed(d_coefs, 5)
    assert np.abs(f_offs - d_offs)[ok].max() <= 1e-3
