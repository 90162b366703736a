"""Synthetic EBSD patterns (uint16) through the C ABI against the FP64 oracle:
integer peaks identical, offsets within the precision's tolerance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


@pytest.fixture(scope="module")
def data512():
    from emida_gb300 import synth
    ref = synth.reference_pattern(512, seed=11)
    pics, _ = synth.deformed_patterns(512, 11, 3, sigma_eps=2e-3)
    return ref, pics


def run(ref, pics, begins, slice_, policy, s, precision, mode, cross=None):
    from emida_gb300 import GpuOffset
    h, w = ref.shape
    cross = cross or (2 * slice_ - 1, 2 * slice_ - 1)
    g = GpuOffset((w, h), begins, (slice_, slice_), cross, len(pics), policy, s, 1, precision,
                  np.uint16, mode)
    g.allocate_memory(ref)
    out = g.get_offset(pics, with_peaks=True)
    assert g.mode == mode
    g.close()
    return out


def well_posed(coefs, s):
    """The fitted extremum lies inside the s x s window.  Outside it the
    quadratic is nearly flat along some direction and the offset is an
    extrapolation whose FP32 error is unbounded (the reference's FP32 path
    shares this; its thesis reports FP32/FP64 outliers of 12.8 %)."""
    b, c, d, e, f = coefs[:, 1], coefs[:, 2], coefs[:, 3], coefs[:, 4], coefs[:, 5]
    y = (b * e - 2 * c * d) / (4 * f * d - e * e)
    x = (-e * y - b) / (2 * d)
    return (x >= 0) & (x <= s - 1) & (y >= 0) & (y <= s - 1)


def assert_offsets(offs, coefs, o_offs, o_coefs, s, tol):
    """Offsets within `tol` for well-posed fits.  For extrapolated fits the
    closed-form extremum amplifies rounding without bound, so there the fitted
    coefficients are compared instead, at the precision's relative level."""
    ok = well_posed(o_coefs, s)
    assert ok.mean() > 0.5  # the tolerance check below must not be vacuous
    err = np.abs(offs - o_offs).max(axis=1)
    assert err[ok].max() <= tol, err[ok].max()
    if (~ok).any():
        rel = 1e-5 if tol >= 1e-6 else 1e-11
        scale = np.abs(o_coefs[~ok]).max(axis=1, keepdims=True)
        assert (np.abs(coefs[~ok] - o_coefs[~ok]) <= rel * scale).all()


def oracle(ref, pics, begins, slice_, policy, s, cross=None):
    from oracle import oracle as eo
    cross = cross or (2 * slice_ - 1, 2 * slice_ - 1)
    pol = eo.POLICY_FFT if policy == "fft" else eo.POLICY_BRUTE
    return eo.get_offsets(ref, pics, begins, slice_, slice_, pol, s, cross[0], cross[1])


def test_brute_double_bit_exact(data512):
    # the brute stages use the oracle's operation order: same bits
    from emida_gb300 import synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 5, 32, margin=40)
    offs, coefs, peaks = run(ref, pics[:2], begins, 64, "brute", 3, "double", "plain")
    o_offs, o_coefs, o_peaks = oracle(ref, pics[:2], begins, 64, "brute", 3)
    assert np.array_equal(peaks, o_peaks)
    assert np.array_equal(offs, o_offs)
    assert np.array_equal(coefs, o_coefs)


@pytest.mark.parametrize("mode", ["plain", "fused"])
@pytest.mark.parametrize("precision,tol", [("double", 1e-9), ("float", 1e-3)])
@pytest.mark.parametrize("s", [3, 5, 7, 9])
def test_fft_vs_oracle(data512, mode, precision, tol, s):
    from emida_gb300 import synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 4, 32, margin=40)
    offs, coefs, peaks = run(ref, pics, begins, 64, "fft", s, precision, mode)
    o_offs, o_coefs, o_peaks = oracle(ref, pics, begins, 64, "fft", s)
    assert np.array_equal(peaks, o_peaks)
    assert_offsets(offs, coefs, o_offs, o_coefs, s, tol)
    assert np.allclose(coefs, o_coefs, rtol=1e-5 if precision == "float" else 1e-11,
                       atol=1e-6 * np.abs(o_coefs).max())


@pytest.mark.parametrize("precision,tol", [("double", 1e-9), ("float", 1e-3)])
def test_fused_radius16(data512, precision, tol):
    # 32 x 32 ROIs: 64-point transforms
    from emida_gb300 import synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 6, 16, margin=30)
    offs, coefs, peaks = run(ref, pics, begins, 32, "fft", 3, precision, "fused")
    o_offs, o_coefs, o_peaks = oracle(ref, pics, begins, 32, "fft", 3)
    assert np.array_equal(peaks, o_peaks)
    assert_offsets(offs, coefs, o_offs, o_coefs, 3, tol)


@pytest.mark.parametrize("radius,precision,tol", [(24, "float", 1e-3), (24, "double", 1e-9),
                                                  (48, "float", 1e-3)])
def test_fused_radius24_48(data512, radius, precision, tol):
    # 48 x 48 ROIs (96-point transforms, 4-lane groups with radix-3 DFTs) and
    # 96 x 96 ROIs (192-point transforms, FP32 only)
    from emida_gb300 import synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 4, radius, margin=radius + 8)
    side = 2 * radius
    offs, coefs, peaks = run(ref, pics[:2], begins, side, "fft", 5, precision, "fused")
    o_offs, o_coefs, o_peaks = oracle(ref, pics[:2], begins, side, "fft", 5)
    assert np.array_equal(peaks, o_peaks)
    assert_offsets(offs, coefs, o_offs, o_coefs, 5, tol)
    p = run(ref, pics[:2], begins, side, "fft", 5, precision, "plain")
    assert np.array_equal(p[2], o_peaks)


@pytest.mark.parametrize("side,precision,tol", [(40, "float", 1e-3), (40, "double", 1e-9),
                                                (50, "float", 1e-3), (76, "float", 1e-3),
                                                (58, "double", 1e-9)])
def test_fused_zero_padded_sides(data512, side, precision, tol):
    # ROI sides whose 2*side is not a fused length are zero-padded into the next
    # one (96, 128, 192): every lag of the 2*side-1 window is unchanged, and the
    # peak index is reported in the reference's 2*side map.
    from emida_gb300 import synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 4, side // 2, margin=side // 2 + 8)
    offs, coefs, peaks = run(ref, pics[:2], begins, side, "fft", 5, precision, "fused")
    o_offs, o_coefs, o_peaks = oracle(ref, pics[:2], begins, side, "fft", 5)
    assert np.array_equal(peaks, o_peaks)
    assert_offsets(offs, coefs, o_offs, o_coefs, 5, tol)
    p = run(ref, pics[:2], begins, side, "fft", 5, precision, "plain")
    assert np.array_equal(p[2], o_peaks)


@pytest.mark.parametrize("side", [128, 100, 116])
def test_fused_256_point_cluster_kernel(data512, side):
    # ROI sides 98..128 (FP32, uint16) run 256-point transforms on a cluster of
    # two CTAs that split the half spectrum; 100 and 116 are zero-padded
    from emida_gb300 import synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 3, side // 2, margin=side // 2 + 8)
    offs, coefs, peaks = run(ref, pics[:3], begins, side, "fft", 5, "float", "fused")
    o_offs, o_coefs, o_peaks = oracle(ref, pics[:3], begins, side, "fft", 5)
    assert np.array_equal(peaks, o_peaks)
    assert_offsets(offs, coefs, o_offs, o_coefs, 5, 1e-3)
    p = run(ref, pics[:3], begins, side, "fft", 5, "float", "plain")
    assert np.array_equal(p[2], o_peaks)


def test_fused_256_many_pairs_and_border_rois(data512):
    # more pairs than clusters (each cluster walks several), ROIs at the
    # borders, x not a multiple of 8, and a repeat that must give the same bits
    ref, pics = data512
    begins = np.array([(0, 0), (384, 0), (0, 384), (384, 384), (3, 5), (201, 77), (383, 13)] * 4,
                      dtype=np.uint32)
    f = run(ref, pics, begins, 128, "fft", 3, "float", "fused")
    g = run(ref, pics, begins, 128, "fft", 3, "float", "fused")
    assert all(np.array_equal(x, y) for x, y in zip(f, g))
    o = oracle(ref, pics, begins[:7], 128, "fft", 3)
    per = len(begins)
    for p in range(len(pics)):
        assert np.array_equal(f[2][p * per:p * per + 7], o[2][p * 7:(p + 1) * 7])


def test_fused_equals_plain_peaks_and_border_rois(data512):
    # ROIs touching every border and with x not a multiple of 8 (TMA x rounding)
    ref, pics = data512
    begins = np.array([(0, 0), (448, 0), (0, 448), (448, 448), (3, 5), (101, 77), (447, 13)],
                      dtype=np.uint32)
    for precision in ("float", "double"):
        f = run(ref, pics, begins, 64, "fft", 3, precision, "fused")
        p = run(ref, pics, begins, 64, "fft", 3, precision, "plain")
        o = oracle(ref, pics, begins, 64, "fft", 3)
        assert np.array_equal(f[2], o[2]) and np.array_equal(p[2], o[2])
        tol = 1e-3 if precision == "float" else 1e-9
        assert_offsets(f[0], f[1], o[0], o[1], 3, tol)
        assert_offsets(p[0], p[1], o[0], o[1], 3, tol)


def test_width_not_multiple_of_8_uses_plain_loads():
    from emida_gb300 import synth
    ref = synth.reference_pattern((300, 260), seed=5)
    pics, _ = synth.deformed_patterns((300, 260), 5, 2)
    begins = np.array([(0, 0), (236, 196), (117, 61)], dtype=np.uint32)
    f = run(ref, pics, begins, 64, "fft", 5, "float", "fused")
    o = oracle(ref, pics, begins, 64, "fft", 5)
    assert np.array_equal(f[2], o[2])
    assert_offsets(f[0], f[1], o[0], o[1], 5, 1e-3)


def test_constant_roi_gives_nan_like_reference():
    # A flat ROI: zero map, peak at index 0, singular fit -> NaN offsets
    # (the reference prints them normalised, src/process_files.hpp:249-253)
    ref = np.full((256, 256), 1000, dtype=np.uint16)
    pics = np.full((1, 256, 256), 1000, dtype=np.uint16)
    begins = np.array([(10, 10)], dtype=np.uint32)
    for mode in ("plain", "fused"):
        offs, _, peaks = run(ref, pics, begins, 64, "fft", 3, "float", mode)
        assert peaks[0] == 0
        assert np.isnan(offs).all()


def test_brute_small_cross_window(data512):
    # --crosssize smaller than 2*slice-1 (src/args_parser.cpp:192-201)
    from emida_gb300 import synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 3, 32, margin=40)
    for cross in ((15, 15), (9, 13)):
        offs, _, peaks = run(ref, pics[:1], begins, 64, "brute", 3, "double", "plain", cross)
        o_offs, _, o_peaks = oracle(ref, pics[:1], begins, 64, "brute", 3, cross)
        assert np.array_equal(peaks, o_peaks)
        assert np.array_equal(offs, o_offs)


def test_repeatable(data512):
    from emida_gb300 import synth
    ref, pics = data512
    _, begins = synth.roi_grid(512, 4, 32, margin=40)
    a = run(ref, pics, begins, 64, "fft", 5, "float", "fused")
    b = run(ref, pics, begins, 64, "fft", 5, "float", "fused")
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


def test_brute_more_pairs_than_one_launch_holds():
    # 256 ROIs x 260 patterns = 66,560 pairs: the brute correlation runs in
    # launches of at most 65,535 pairs, and the pairs past the first launch
    # keep the oracle's bits
    from emida_gb300 import synth
    ref = synth.reference_pattern(128, seed=13)
    base, _ = synth.deformed_patterns(128, 13, 4, sigma_eps=2e-3)
    pics = np.ascontiguousarray(base[np.arange(260) % 4])
    begins = [(x, y) for y in range(0, 121, 8) for x in range(0, 121, 8)]
    offs, coefs, peaks = run(ref, pics, begins, 8, "brute", 3, "double", "plain", (15, 15))
    n = len(begins)
    o_offs, o_coefs, o_peaks = oracle(ref, pics[-4:], begins, 8, "brute", 3, (15, 15))
    assert np.array_equal(peaks[-4 * n:], o_peaks)
    assert np.array_equal(offs[-4 * n:], o_offs)
    assert np.array_equal(coefs[-4 * n:], o_coefs)
    # and every repeat of a pattern gives its first result
    first = offs[:4 * n].reshape(4, n, 2)
    assert np.array_equal(offs.reshape(260, n, 2), first[np.arange(260) % 4])
