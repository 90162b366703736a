"""Per-stage kernels through the C ABI's launchers (src/kernels.cuh:56-125),
against the reference's unit-test vectors (test/*.cpp) and the oracle."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu

DOUBLE, FLOAT = 0, 1


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build_library()


def dev(a):
    from emida_gb300 import DeviceBuffer
    return DeviceBuffer.from_array(np.ascontiguousarray(a))


def empty(nbytes):
    from emida_gb300 import DeviceBuffer
    b = DeviceBuffer(nbytes)
    b.zero()
    return b


def call(name, *args):
    """Device buffers are passed as DeviceBuffer objects: the argument tuple
    keeps them (and their device memory) alive until the launch has finished."""
    from emida_gb300 import DeviceBuffer, _lib
    _lib.call(name, *[a.ptr if isinstance(a, DeviceBuffer) else a for a in args])


def sums(pics, begins, sw, sh):
    pics = np.ascontiguousarray(pics)
    b, h, w = pics.shape
    begins = np.asarray(begins, dtype=np.uint32)
    in_type = 0 if pics.dtype == np.uint16 else 1
    dt = np.uint32 if in_type == 0 else np.float64
    out = empty(len(begins) * b * 8)
    db = dev(begins)
    call("emida_gb_run_sum", dev(pics), in_type, w, h, db, len(begins), sw, sh, b, out)
    return out.download(dt, len(begins) * b)


def test_sum_kats():
    # test/sum_test.cpp:58-66, :113-149
    v = np.array([[1, 3, 5, 8], [8, 10, 4, 1], [3, 2, 5, 15]], dtype=np.float64)[None]
    assert list(sums(v, [(0, 0), (1, 1)], 2, 2)) == [22, 21]
    for (sw, sh), (w, h), begins, b in [((29, 40), (31, 43), [(0, 0), (1, 1)], 1),
                                        ((32, 32), (64, 64), [(0, 0), (0, 16), (16, 16), (32, 32)], 1),
                                        ((32, 32), (64, 64), [(0, 0), (0, 16), (16, 16), (32, 32)], 97),
                                        ((21, 41), (23, 43), [(0, 0), (1, 1)], 8)]:
        data = np.arange(w * h * b, dtype=np.float64).reshape(b, h, w)
        exp = [data[k, y:y + sh, x:x + sw].sum() for k in range(b) for (x, y) in begins]
        assert np.array_equal(sums(data, begins, sw, sh), exp)


def test_sum_u16_exact_and_wrapping():
    from oracle import oracle as eo
    rng = np.random.default_rng(1)
    pics = rng.integers(0, 65536, size=(3, 300, 300), dtype=np.uint16)
    begins = [(0, 0), (17, 33), (236, 236)]
    assert np.array_equal(sums(pics, begins, 64, 64), eo.roi_sums(pics, begins, 64, 64))
    big = np.full((1, 300, 300), 65535, dtype=np.uint16)
    assert sums(big, [(0, 0)], 300, 300)[0] == (65535 * 90000) % (1 << 32)


def prepare(pics, begins, sw, sh, out_w, out_h, sums_arr, wx, wy, precision):
    pics = np.ascontiguousarray(pics)
    b, h, w = pics.shape
    in_type = 0 if pics.dtype == np.uint16 else 1
    T = np.float64 if precision == DOUBLE else np.float32
    out = empty(len(begins) * b * out_w * out_h * np.dtype(T).itemsize)
    hann = np.concatenate([np.asarray(wx, T), np.asarray(wy, T)])
    call("emida_gb_run_prepare", dev(pics), in_type, precision, out, dev(hann),
         dev(np.asarray(sums_arr)), dev(np.asarray(begins, np.uint32)), w, h, sw, sh,
         out_w, out_h, len(begins), b)
    return out.download(T, (len(begins) * b, out_h, out_w))


def test_prepare_kats():
    # test/prepare_test.cpp:47-210
    pic = np.arange(1, 31, dtype=np.uint16).reshape(1, 5, 6)
    begins = [(1, 2), (0, 1)]
    s = sums(pic, begins, 5, 3)
    exp = np.array([[-8, -7, -6, -5, -4], [-2, -1, 0, 1, 2], [4, 5, 6, 7, 8]], dtype=float)
    out = prepare(pic, begins, 5, 3, 5, 3, s, np.ones(5), np.ones(3), DOUBLE)
    assert np.array_equal(out[0], exp) and np.array_equal(out[1], exp)
    wx, wy = np.ones(5), np.ones(3)
    wx[2], wy[1] = 0.5, 0.25
    out = prepare(pic, begins, 5, 3, 5, 3, s, wx, wy, DOUBLE)
    assert np.array_equal(out[0], [[-8, -7, -3, -5, -4], [-0.5, -0.25, 0, 0.25, 0.5], [4, 5, 3, 7, 8]])
    out = prepare(pic, begins, 5, 3, 10, 6, s, np.ones(5), np.ones(3), DOUBLE)
    assert np.array_equal(out[0, :3, :5], exp) and not out[0, 3:].any() and not out[0, :, 5:].any()
    # batch: test/prepare_test.cpp:80-125 (sums given as in the test)
    pic2 = np.concatenate([pic, pic[:, ::-1, :]], 0)
    out = prepare(pic2, begins, 5, 3, 5, 3, np.array([330, 225, 0, 0], np.uint32), np.ones(5),
                  np.ones(3), DOUBLE)
    assert np.array_equal(out[2], [[14, 15, 16, 17, 18], [8, 9, 10, 11, 12], [2, 3, 4, 5, 6]])


def test_prepare_f32_bit_exact():
    from oracle import oracle as eo
    rng = np.random.default_rng(2)
    pics = rng.integers(0, 4096, size=(2, 200, 200), dtype=np.uint16)
    begins = [(0, 0), (13, 71), (136, 136)]
    s = sums(pics, begins, 64, 64)
    hx = eo.hanning(64).astype(np.float32)
    got = prepare(pics, begins, 64, 64, 128, 128, s, hx, hx, FLOAT)
    exp = eo.prepare_f32(pics, begins, 64, 64, 128, 128, s, hx, hx)
    assert np.array_equal(got, exp)
    s64 = s.astype(np.float64)
    got = prepare(pics, begins, 64, 64, 64, 64, s, eo.hanning(64), eo.hanning(64), DOUBLE)
    assert np.array_equal(got, eo.prepare_f64(pics, begins, 64, 64, 64, 64, s64, eo.hanning(64), eo.hanning(64)))


def xcorr(a, b, w, h, rw, rh, ref_slices, batch, precision):
    T = np.float64 if precision == DOUBLE else np.float32
    a = np.ascontiguousarray(a, T)
    b = np.ascontiguousarray(b, T)
    out = empty(ref_slices * batch * rw * rh * np.dtype(T).itemsize)
    call("emida_gb_run_cross_corr", dev(a), dev(b), out, precision, w, h, rw, rh,
         ref_slices, batch)
    return out.download(T, (ref_slices * batch, rh, rw))


@pytest.mark.parametrize("precision", [DOUBLE, FLOAT])
def test_cross_corr_kats(precision):
    # test/cross_corr_test.cpp:17-218 (integer-valued data: exact in both precisions)
    a = np.arange(1, 10).reshape(3, 3)
    assert np.array_equal(xcorr(a, a, 3, 3, 5, 5, 1, 1, precision)[0],
                          [[9, 26, 50, 38, 21], [42, 94, 154, 106, 54], [90, 186, 285, 186, 90],
                           [54, 106, 154, 94, 42], [21, 38, 50, 26, 9]])
    assert np.array_equal(xcorr(a, a, 3, 3, 3, 3, 1, 1, precision)[0],
                          [[94, 154, 106], [186, 285, 186], [106, 154, 94]])
    a = np.array([[1, 2, 3, 4], [5, 6, 7, 8], [9, 10, 11, 12], [3, 2, 1, 4], [2, 6, 10, 8], [9, 8, 11, 5]])
    b = np.array([[8, 7, 6, 5], [16, 15, 14, 13], [4, 3, 2, 1], [1, 2, 3, 4], [16, 5, 14, 13], [8, 3, 2, 1]])
    res = xcorr(a, b, 4, 3, 7, 5, 2, 1, precision)
    assert np.array_equal(res[0], [[1, 4, 10, 20, 25, 24, 16], [18, 56, 116, 200, 194, 160, 96],
                                   [79, 192, 342, 532, 471, 364, 208], [142, 316, 524, 768, 638, 468, 256],
                                   [45, 104, 178, 268, 229, 172, 96]])
    assert np.array_equal(res[1], [[3, 8, 14, 36, 27, 20, 32], [41, 78, 84, 186, 187, 140, 128],
                                   [47, 149, 294, 455, 381, 312, 172], [125, 260, 362, 479, 303, 227, 88],
                                   [36, 59, 86, 78, 45, 21, 5]])
    res = xcorr(a, b, 4, 3, 5, 5, 2, 1, precision)
    assert np.array_equal(res[1], [[8, 14, 36, 27, 20], [78, 84, 186, 187, 140], [149, 294, 455, 381, 312],
                                   [260, 362, 479, 303, 227], [59, 86, 78, 45, 21]])


def test_cross_corr_64_fixture():
    # test/cross_corr_test.cpp:207-218 with test/res/cross_corr/64_*.txt
    cc = np.load(os.path.join(GOLDEN, "cross_corr_64.npz"))
    res = xcorr(cc["A"], cc["B"], 64, 64, 127, 127, 1, 1, DOUBLE)
    assert np.array_equal(res[0], cc["res"])


def test_cross_corr_batched_refs_bit_exact():
    from oracle import oracle as eo
    rng = np.random.default_rng(4)
    pics = rng.normal(size=(6, 20, 24))
    refs = rng.normal(size=(3, 20, 24))
    got = xcorr(pics, refs, 24, 20, 31, 25, 3, 2, DOUBLE)
    assert np.array_equal(got, eo.cross_corr_brute(pics, refs, 31, 25, 3))


@pytest.mark.parametrize("w2,h2", [(128, 128), (64, 64), (96, 96), (8, 8), (12, 10), (256, 256)])
def test_fft_r2c_c2r_against_numpy(w2, h2):
    rng = np.random.default_rng(w2 * 1000 + h2)
    maps = 3
    x = rng.normal(size=(maps, h2, w2))
    half = w2 // 2 + 1
    spec = empty(maps * h2 * half * 16)
    call("emida_gb_run_fft_r2c", dev(x), spec, maps, w2, h2, DOUBLE)
    got = spec.download(np.complex128, (maps, h2, half))
    exp = np.fft.rfft2(x)
    assert np.abs(got - exp).max() <= 1e-10 * np.abs(exp).max()
    out = empty(maps * h2 * w2 * 8)
    call("emida_gb_run_fft_c2r", spec, out, maps, w2, h2, DOUBLE)
    back = out.download(np.float64, (maps, h2, w2))
    assert np.abs(back - x * w2 * h2).max() <= 1e-10 * np.abs(x).max() * w2 * h2


def test_fft_float():
    rng = np.random.default_rng(5)
    x = rng.normal(size=(2, 128, 128)).astype(np.float32)
    spec = empty(2 * 128 * 65 * 8)
    call("emida_gb_run_fft_r2c", dev(x), spec, 2, 128, 128, FLOAT)
    got = spec.download(np.complex64, (2, 128, 65))
    exp = np.fft.rfft2(x.astype(np.float64))
    assert np.abs(got - exp).max() <= 1e-5 * np.abs(exp).max()


def test_hadamard():
    # src/hadamard.cu:39-40: P * conj(R), R indexed modulo one_area * ref_slices
    rng = np.random.default_rng(6)
    P = (rng.normal(size=(2, 3, 10)) + 1j * rng.normal(size=(2, 3, 10))).astype(np.complex128)
    R = (rng.normal(size=(3, 10)) + 1j * rng.normal(size=(3, 10))).astype(np.complex128)
    d = dev(P)
    call("emida_gb_run_hadamard", d, dev(R), 10, 3, 2, DOUBLE)
    got = d.download(np.complex128, P.shape)
    assert np.allclose(got, P * np.conj(R)[None], rtol=1e-15, atol=0)


def maxarg(data, size, n, precision=DOUBLE):
    from emida_gb300 import DATA_INDEX_F32, DATA_INDEX_F64
    T = np.float64 if precision == DOUBLE else np.float32
    dt = DATA_INDEX_F64 if precision == DOUBLE else DATA_INDEX_F32
    out = empty(n * dt.itemsize)
    call("emida_gb_run_maxarg", dev(np.asarray(data, T)), size, n, out, precision)
    return out.download(dt, n)


def test_maxarg_kats():
    # test/maxarg_test.cpp:63-231
    r = maxarg([1, 3, 5, 8, 10, 4, 3, 2], 8, 1)
    assert (r[0]["data"], r[0]["index"]) == (10, 4)
    v = [1, 3, 0, 8, 10, 4, 0, 3, 0, 0, 0, 0, 1, 1, 0, 1]
    r = maxarg(v + v, 16, 2)
    assert [(x["data"], x["index"]) for x in r] == [(10, 4), (10, 4)]
    r = maxarg([1, 3, 5, 8, 10, 4, 3, 2, 1, 12, 15, 18, 10, 4, 3, 2], 8, 2)
    assert [(x["data"], x["index"]) for x in r] == [(10, 4), (18, 3)]
    data = []
    mom = 0.0
    for _ in range(4096):
        data.append(mom)
        mom += 0.007
        if mom > 1:
            mom = -2
    d = np.array(data)
    a = d[:1333].copy()
    a[1001] = 3
    r = maxarg(a, 1333, 1)
    assert (r[0]["data"], r[0]["index"]) == (3, 1001)
    b = d[:3999].copy()
    b[1001], b[1024], b[1333], b[3000] = 3, 4, 4, 4
    r = maxarg(b, 1333, 3)
    assert [(x["data"], x["index"]) for x in r] == [(4, 1024), (4, 0), (4, 334)]
    c = d.copy()
    c[1024] = 3
    r = maxarg(c, 4096, 1)
    assert (r[0]["data"], r[0]["index"]) == (3, 1024)


@pytest.mark.parametrize("precision", [DOUBLE, FLOAT])
def test_maxarg_first_maximum_on_ties(precision):
    m = np.zeros((2, 16384))
    m[0, [9000, 77, 16000]] = 5
    m[1, :] = -1
    r = maxarg(m, 16384, 2, precision)
    assert list(r["index"]) == [77, 0]


def extract(data, maxes_idx, s, cw, ch, n, policy, precision=DOUBLE):
    from emida_gb300 import DATA_INDEX_F32, DATA_INDEX_F64
    T = np.float64 if precision == DOUBLE else np.float32
    dt = DATA_INDEX_F64 if precision == DOUBLE else DATA_INDEX_F32
    mi = np.zeros(n, dtype=dt)
    mi["index"] = maxes_idx
    out = empty(n * s * s * np.dtype(T).itemsize)
    call("emida_gb_run_extract_neighbors", dev(np.asarray(data, T)), dev(mi), out, s,
         cw, ch, n, policy, precision)
    return out.download(T, (n, s * s))


def test_extract_kats():
    # test/maxarg_test.cpp:8-61
    assert np.array_equal(extract(np.arange(25), [18], 3, 5, 5, 1, 0)[0],
                          [12, 13, 14, 17, 18, 19, 22, 23, 24])
    got = extract(np.arange(50), [18, 6], 3, 5, 5, 2, 0)
    assert np.array_equal(got.ravel(), [12, 13, 14, 17, 18, 19, 22, 23, 24, 25, 26, 27, 30, 31, 32, 35, 36, 37])


@pytest.mark.parametrize("policy", [0, 1])
@pytest.mark.parametrize("s", [3, 5, 9])
def test_extract_matches_oracle_with_clamps(policy, s):
    # peaks on every border, including the reference's inclusive [0, cross] clamp
    from oracle import oracle as eo
    rng = np.random.default_rng(7)
    cw = ch = 15
    size = cw * ch if policy == 0 else (cw + 1) * (ch + 1)
    n = 12
    maps = rng.normal(size=(n, size))
    idx = np.array([0, size - 1, 7, size // 2, cw - 1, cw, 3 * (cw + policy), size - 2, 1, 100, 200, 31],
                   dtype=np.uint32) % size
    got = extract(maps, idx, s, cw, ch, n, policy)
    exp = eo.extract_neighbors(maps, idx, policy, cw, ch, s)
    assert np.array_equal(got, exp)
