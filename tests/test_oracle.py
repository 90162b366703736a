"""The oracle (oracle/emida_oracle.c) pinned against the reference's own golden
vectors and against outputs of the reference's CPU code (tests/golden/).
CPU only."""
import json
import os

import numpy as np
import pytest

from oracle import oracle as eo
from tests.conftest import GOLDEN

EXPECTED = json.load(open(os.path.join(GOLDEN, "get_offset_expected.json")))
REF_OUT = np.load(os.path.join(GOLDEN, "ref_cpu_outputs.npz"))


def golden_pair():
    return np.load(os.path.join(GOLDEN, "data_pic.npy")), np.load(os.path.join(GOLDEN, "data_temp.npy"))


def slice_begins(src, size, step):
    """src/slice_picture.hpp:87-97 get_slice_begins, (x, y), x fastest."""
    return [(x, y) for y in range(0, src - size + 1, step) for x in range(0, src - size + 1, step)]


def test_get_offset_single_roi():
    # test/get_offset_test.cpp:10-27: one 64x64 ROI, brute, 127 lags, s = 3
    pic, temp = golden_pair()
    offs, _, _ = eo.get_offsets(temp[:64, :64], pic[None, :64, :64], [(0, 0)], 64, 64,
                                eo.POLICY_BRUTE, 3, 127, 127)
    g = EXPECTED["get_offset_single"]
    assert abs(offs[0, 0] - g["x"]) <= g["tol"]
    assert abs(offs[0, 1] - g["y"]) <= g["tol"]


@pytest.mark.parametrize("policy", [eo.POLICY_BRUTE, eo.POLICY_FFT])
@pytest.mark.parametrize("batch", [1, 5])
def test_get_offset_batched(policy, batch):
    # test/get_offset_test.cpp:120-200: 49 ROIs, step 32, tolerance 7e-13
    pic, temp = golden_pair()
    g = EXPECTED["get_offset_batched"]
    exp = np.tile(np.array(g["offsets"]), (batch, 1))
    offs, _, _ = eo.get_offsets(temp, np.repeat(pic[None], batch, 0), slice_begins(256, 64, 32),
                                64, 64, policy, 3, 127, 127)
    assert np.abs(offs - exp).max() <= g["tol"]


@pytest.mark.parametrize("s", [3, 5, 7, 9])
def test_lstsq_tables_match_reference(s):
    # src/subpixel_max.cpp:22-58, bit for bit
    assert np.array_equal(eo.lstsq_matrix(s).ravel(), REF_OUT[f"lstsq_{s}"])


@pytest.mark.parametrize("s", [3, 5, 7, 9])
def test_fit_matches_reference(s):
    sub, co = eo.subpixel_max(REF_OUT[f"fit_{s}_neigh"], s)
    assert np.array_equal(sub, REF_OUT[f"fit_{s}_sub"])
    assert np.array_equal(co, REF_OUT[f"fit_{s}_coefs"])


def test_hanning():
    # test/prepare_test.cpp:18-23 and the reference's generate_hanning at 64
    # EXPECT_DOUBLE_EQ: within 4 ulps; cos(pi/2) is not exactly 0 in FP64
    assert np.allclose(eo.hanning(5), [0, 0.5, 1, 0.5, 0], rtol=4 * 2.2e-16, atol=1e-16)
    assert np.array_equal(eo.hanning(64), REF_OUT["hann_64"])


@pytest.mark.parametrize("key", ["xcorr_16x12_31x23", "xcorr_9x9_5x7"])
def test_brute_matches_reference_serial(key):
    res = REF_OUT[key + "_res"]
    out = eo.cross_corr_brute(REF_OUT[key + "_pics"], REF_OUT[key + "_refs"], res.shape[2], res.shape[1])
    assert np.array_equal(out, res)


def test_brute_kats():
    # test/cross_corr_test.cpp:17-150
    a = np.arange(1, 10, dtype=float).reshape(1, 3, 3)
    exp = [[9, 26, 50, 38, 21], [42, 94, 154, 106, 54], [90, 186, 285, 186, 90],
           [54, 106, 154, 94, 42], [21, 38, 50, 26, 9]]
    assert np.array_equal(eo.cross_corr_brute(a, a, 5, 5)[0], exp)
    assert np.array_equal(eo.cross_corr_brute(a, a, 3, 3)[0], [[94, 154, 106], [186, 285, 186], [106, 154, 94]])
    a = np.arange(1, 13, dtype=float).reshape(1, 3, 4)
    b = np.array([[8, 7, 6, 5], [16, 15, 14, 13], [4, 3, 2, 1]], dtype=float)[None]
    exp = [[1, 4, 10, 20, 25, 24, 16], [18, 56, 116, 200, 194, 160, 96],
           [79, 192, 342, 532, 471, 364, 208], [142, 316, 524, 768, 638, 468, 256],
           [45, 104, 178, 268, 229, 172, 96]]
    assert np.array_equal(eo.cross_corr_brute(a, b, 7, 5)[0], exp)
    cc = np.load(os.path.join(GOLDEN, "cross_corr_64.npz"))
    assert np.array_equal(eo.cross_corr_brute(cc["A"][None].astype(float), cc["B"][None].astype(float),
                                              127, 127)[0], cc["res"])


def test_fft_policy_equals_brute_on_lags():
    rng = np.random.default_rng(3)
    p = np.zeros((16, 16))
    r = np.zeros((16, 16))
    p[:8, :8] = rng.normal(size=(8, 8))
    r[:8, :8] = rng.normal(size=(8, 8))
    fft = eo.cross_corr_fft(p, r)
    brute = eo.cross_corr_brute(p[None, :8, :8], r[None, :8, :8], 15, 15)[0]
    # FFT index of lag (sx, sy) is (sx mod 16, sy mod 16) (src/kernels.cuh:36-53);
    # the inverse is unnormalised like cuFFT's C2R, so values carry a 16*16 factor
    for sy in range(-7, 8):
        for sx in range(-7, 8):
            assert abs(fft[sy % 16, sx % 16] / 256 - brute[sy + 7, sx + 7]) < 1e-12
    assert np.abs(fft[8, :]).max() < 1e-9 and np.abs(fft[:, 8]).max() < 1e-9


def test_maxarg_and_extract_kats():
    # test/maxarg_test.cpp:8-100
    v = np.arange(25, dtype=float)[None]
    n = eo.extract_neighbors(v, [18], eo.POLICY_BRUTE, 5, 5, 3)
    assert np.array_equal(n[0], [12, 13, 14, 17, 18, 19, 22, 23, 24])
    v = np.arange(50, dtype=float).reshape(2, 25)
    n = eo.extract_neighbors(v, [18, 6], eo.POLICY_BRUTE, 5, 5, 3)
    assert np.array_equal(n.ravel(), [12, 13, 14, 17, 18, 19, 22, 23, 24, 25, 26, 27, 30, 31, 32, 35, 36, 37])
    idx, val = eo.maxarg(np.array([[1, 3, 5, 8, 10, 4, 3, 2]], dtype=float))
    assert (idx[0], val[0]) == (4, 10)
    data = []
    mom = 0.0
    for _ in range(3999):
        data.append(mom)
        mom += 0.007
        if mom > 1:
            mom = -2
    data = np.array(data)
    data[1001], data[1024], data[1333], data[3000] = 3, 4, 4, 4
    idx, val = eo.maxarg(data.reshape(3, 1333))
    assert list(idx) == [1024, 0, 334] and list(val) == [4, 4, 4]


def test_first_maximum_tie_rule():
    m = np.zeros((1, 20))
    m[0, [3, 7, 11]] = 5
    idx, _ = eo.maxarg(m)
    assert idx[0] == 3


def test_prepare_kats():
    # test/prepare_test.cpp:47-161
    pic = np.arange(1, 31, dtype=np.uint16).reshape(1, 5, 6)
    begins = [(1, 2), (0, 1)]
    sums = eo.roi_sums(pic, begins, 5, 3)
    out = eo.prepare_f64(pic, begins, 5, 3, 5, 3, sums.astype(float), np.ones(5), np.ones(3))
    exp = [[-8, -7, -6, -5, -4], [-2, -1, 0, 1, 2], [4, 5, 6, 7, 8]]
    assert np.array_equal(out[0], exp) and np.array_equal(out[1], exp)
    wx, wy = np.ones(5), np.ones(3)
    wx[2], wy[1] = 0.5, 0.25
    out = eo.prepare_f64(pic, begins, 5, 3, 5, 3, sums.astype(float), wx, wy)
    assert np.array_equal(out[0], [[-8, -7, -3, -5, -4], [-0.5, -0.25, 0, 0.25, 0.5], [4, 5, 3, 7, 8]])
    out = eo.prepare_f64(pic, begins, 5, 3, 10, 6, sums.astype(float), np.ones(5), np.ones(3))
    assert np.array_equal(out[0, :3, :5], exp) and not out[0, 3:].any() and not out[0, :, 5:].any()


def test_hann_window_fixture():
    # test/res/hann/5_{A,res}.txt: the 5x5 slice times hx[x] * hy[y]
    h = np.load(os.path.join(GOLDEN, "hann_5.npz"))
    w = eo.hanning(5)
    assert np.allclose(h["A"] * w[None, :] * w[:, None], h["res"], rtol=0, atol=1e-12)


def test_sums_kats():
    # test/sum_test.cpp:44-149
    v = np.array([[1, 3, 5, 8], [8, 10, 4, 1], [3, 2, 5, 15]], dtype=np.uint16)[None]
    assert list(eo.roi_sums(v, [(0, 0), (1, 1)], 2, 2)) == [22, 21]
    for (sw, sh), (w, hh), begins, b in [((29, 40), (31, 43), [(0, 0), (1, 1)], 1),
                                          ((32, 32), (64, 64), [(0, 0), (0, 16), (16, 16), (32, 32)], 97),
                                          ((21, 41), (23, 43), [(0, 0), (1, 1)], 8)]:
        data = np.arange(w * hh * b, dtype=np.float64).reshape(b, hh, w)
        exp = []
        for k in range(b):
            for (x, y) in begins:
                exp.append(data[k, y:y + sh, x:x + sw].sum())
        assert np.allclose(eo.roi_sums(data, begins, sw, sh), exp, rtol=0, atol=0)


def test_u16_sum_wraps_like_uint32():
    pic = np.full((1, 300, 300), 65535, dtype=np.uint16)
    s = eo.roi_sums(pic, [(0, 0)], 300, 300)
    assert s[0] == (65535 * 90000) % (1 << 32)


def test_subpixel_kats():
    # test/subpixel_max_test.cpp:21-46
    sub, co = eo.subpixel_max(np.array([1, 2, 3, 4, 5, 6, 7, 8, 9], dtype=float), 3)
    assert np.allclose(co[0], [1, 1, 3, 0, 0, 0], atol=1e-15)
    sub, co = eo.subpixel_max(np.array([1, 2, 3, 7, 9, 8, 4, 5, 6], dtype=float), 3)
    assert np.allclose(co[0], [1.0, 1.833333333333333, 10.5, -0.5, 0, -4.5], rtol=4 * 2.2e-16, atol=1e-15)
    assert sub[0, 0] == pytest.approx(1.8333333333333333, abs=4e-16)
    assert sub[0, 1] == pytest.approx(1.1666666666666666, abs=4e-16)


def test_oracle_fft_matches_numpy():
    rng = np.random.default_rng(9)
    for n in (8, 12, 96, 128, 74):
        x = rng.normal(size=n) + 1j * rng.normal(size=n)
        assert np.abs(eo.fft_c2c(x) - np.fft.fft(x)).max() < 1e-12
        assert np.abs(eo.fft_c2c(x, True) - np.fft.ifft(x) * n).max() < 1e-12


def test_reference_lib_agrees_where_built():
    ref = eo.ref_lib()
    if ref is None:
        pytest.skip("reference CPU code not built on this machine")
    import ctypes
    for s in (3, 5, 7, 9):
        m = np.zeros(6 * s * s)
        assert ref.ref_lstsq_matrix(s, m.ctypes.data_as(ctypes.POINTER(ctypes.c_double))) == 0
        assert np.array_equal(m, eo.lstsq_matrix(s).ravel())


@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("float", 1e-2)])
def test_reference_cpu_brute_path_agrees_with_the_oracle(precision, tol):
    """The reference's own CPU pieces (sums_serial, generate_hanning,
    cross_corr_serial, subpixel_max_serial) through one pattern's ROIs, as the
    CPU baseline runs them, against the oracle's brute path."""
    ref_lib = eo.ref_lib()
    if ref_lib is None:
        pytest.skip("reference CPU code not built on this machine")
    from emida_gb300 import synth
    ref = synth.reference_pattern(256, seed=8)
    pics, _ = synth.deformed_patterns(256, 8, 1, 3e-3)
    _, begins = synth.roi_grid(256, 2, 32, margin=48)
    prep = eo.ref_prepare_reference(ref_lib, ref, begins, 64, precision)
    offs, peaks = eo.ref_brute_pattern(ref_lib, prep, pics[0], begins, 64, 127, 5, precision)
    o_offs, o_coefs, o_peaks = eo.get_offsets(ref, pics, begins, 64, 64, eo.POLICY_BRUTE, 5, 127, 127)
    assert np.array_equal(peaks, o_peaks)
    assert np.abs(offs - o_offs).max() <= tol


def test_homography_fit_matches_reference_script():
    # python/process_offsets.py run on seeded offsets (tests/golden/make_homography_golden.py)
    from oracle import oracle as eo
    g = np.load(os.path.join(GOLDEN, "homography_golden.npz"))
    for off, uu in zip(g["offsets"], g["uu"]):
        got = eo.homography_fit(g["mids"], off, g["centre"])
        assert np.allclose(got, uu, rtol=1e-12, atol=1e-15)
