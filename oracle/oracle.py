"""ctypes front end of the CPU FP64 oracle (oracle/_build/libemida_oracle.so).

TEST INFRASTRUCTURE ONLY: the oracle.  Only tests/, __graft_entry__.smoke()
and bench.py's CPU-baseline / reference arm import this module.  It builds the
library with `make -C oracle oracle` on first use when it is missing.

Every function mirrors one in emida_oracle.h, which cites the reference
file:line it restates.
"""
import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libemida_oracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libemida_ref.so")

POLICY_BRUTE, POLICY_FFT = 0, 1
IN_U16, IN_F64 = 0, 1

_lock = threading.Lock()
_lib = None


class EoParams(ctypes.Structure):
    _fields_ = [
        ("src_w", ctypes.c_uint32), ("src_h", ctypes.c_uint32),
        ("begins", ctypes.POINTER(ctypes.c_uint32)), ("n_rois", ctypes.c_uint32),
        ("slice_w", ctypes.c_uint32), ("slice_h", ctypes.c_uint32),
        ("cross_w", ctypes.c_uint32), ("cross_h", ctypes.c_uint32),
        ("batch", ctypes.c_uint32), ("policy", ctypes.c_int32),
        ("fitsize", ctypes.c_int32), ("in_type", ctypes.c_int32),
    ]


def build():
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                build()
            _lib = ctypes.CDLL(LIB_PATH)
    return _lib


def ref_lib():
    """The reference's own CPU code (oracle/_ref), or None where it was not built."""
    if not os.path.exists(REF_LIB_PATH):
        return None
    return ctypes.CDLL(REF_LIB_PATH)


def ref_brute_pattern(ref_lib, ref_prepared, pattern, begins, slice_, cross, s, precision):
    """One pattern's ROIs through the brute path with the reference's own CPU
    code (oracle/_ref): (offsets [n_rois][2], peaks [n_rois]).  ref_prepared
    comes from ref_prepare_reference in the same precision."""
    pattern = np.ascontiguousarray(pattern, dtype=np.uint16)
    h, w = pattern.shape
    begins = np.ascontiguousarray(begins, dtype=np.uint32).reshape(-1, 2)
    offs = np.zeros((len(begins), 2))
    peaks = np.zeros(len(begins), dtype=np.uint32)
    ct = ctypes.c_float if precision == "float" else ctypes.c_double
    fn = ref_lib.ref_brute_offsets_f32 if precision == "float" else ref_lib.ref_brute_offsets_f64
    fn(_p(pattern, ctypes.c_uint16), _p(ref_prepared, ct), w, h, _p(begins, ctypes.c_uint32),
       len(begins), slice_, cross, s, _p(offs), _p(peaks, ctypes.c_uint32))
    return offs, peaks


def ref_prepare_reference(ref_lib, ref, begins, slice_, precision):
    """The reference ROIs prepared by the reference's CPU pieces (oracle/_ref)."""
    ref = np.ascontiguousarray(ref, dtype=np.uint16)
    h, w = ref.shape
    begins = np.ascontiguousarray(begins, dtype=np.uint32).reshape(-1, 2)
    dt, ct = (np.float32, ctypes.c_float) if precision == "float" else (np.float64, ctypes.c_double)
    out = np.zeros((len(begins), slice_, slice_), dtype=dt)
    fn = ref_lib.ref_prepare_reference_f32 if precision == "float" else ref_lib.ref_prepare_reference_f64
    fn(_p(ref, ctypes.c_uint16), w, h, _p(begins, ctypes.c_uint32), len(begins), slice_, _p(out, ct))
    return out


def _p(a, ct=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def hanning(n):
    out = np.zeros(n)
    lib().eo_hanning(ctypes.c_size_t(n), _p(out))
    return out


def lstsq_matrix(s):
    out = np.zeros(6 * s * s)
    if lib().eo_lstsq_matrix(s, _p(out)) != 0:
        raise ValueError(f"unsupported fit size {s}")
    return out.reshape(6, s * s)


def roi_sums(pics, begins, slice_w, slice_h):
    pics = np.ascontiguousarray(pics)
    b, h, w = pics.shape
    begins = np.ascontiguousarray(begins, dtype=np.uint32).reshape(-1, 2)
    if pics.dtype == np.uint16:
        out = np.zeros(b * len(begins), dtype=np.uint32)
        lib().eo_roi_sums_u16(_p(pics, ctypes.c_uint16), w, h, _p(begins, ctypes.c_uint32),
                              len(begins), slice_w, slice_h, b, _p(out, ctypes.c_uint32))
    else:
        pics = pics.astype(np.float64)
        out = np.zeros(b * len(begins))
        lib().eo_roi_sums_f64(_p(pics), w, h, _p(begins, ctypes.c_uint32), len(begins),
                              slice_w, slice_h, b, _p(out))
    return out


def prepare_f64(pics, begins, slice_w, slice_h, out_w, out_h, sums, hx, hy):
    pics = np.ascontiguousarray(pics)
    b, h, w = pics.shape
    begins = np.ascontiguousarray(begins, dtype=np.uint32).reshape(-1, 2)
    in_type = IN_U16 if pics.dtype == np.uint16 else IN_F64
    if in_type == IN_F64:
        pics = pics.astype(np.float64)
    out = np.zeros((b * len(begins), out_h, out_w))
    sums = np.ascontiguousarray(sums, dtype=np.float64)
    hx = np.ascontiguousarray(hx, dtype=np.float64)
    hy = np.ascontiguousarray(hy, dtype=np.float64)
    lib().eo_prepare_f64(pics.ctypes.data_as(ctypes.c_void_p), in_type, w, h,
                         _p(begins, ctypes.c_uint32), len(begins), slice_w, slice_h, out_w,
                         out_h, b, _p(sums), _p(hx), _p(hy), _p(out))
    return out


def prepare_f32(pics, begins, slice_w, slice_h, out_w, out_h, sums_u32, hx, hy):
    pics = np.ascontiguousarray(pics, dtype=np.uint16)
    b, h, w = pics.shape
    begins = np.ascontiguousarray(begins, dtype=np.uint32).reshape(-1, 2)
    out = np.zeros((b * len(begins), out_h, out_w), dtype=np.float32)
    sums = np.ascontiguousarray(sums_u32, dtype=np.uint32)
    hx = np.ascontiguousarray(hx, dtype=np.float32)
    hy = np.ascontiguousarray(hy, dtype=np.float32)
    lib().eo_prepare_f32(_p(pics, ctypes.c_uint16), w, h, _p(begins, ctypes.c_uint32),
                         len(begins), slice_w, slice_h, out_w, out_h, b,
                         _p(sums, ctypes.c_uint32), _p(hx, ctypes.c_float),
                         _p(hy, ctypes.c_float), _p(out, ctypes.c_float))
    return out


def cross_corr_brute(pics, refs, res_w, res_h, ref_slices=None):
    pics = np.ascontiguousarray(pics, dtype=np.float64)
    refs = np.ascontiguousarray(refs, dtype=np.float64)
    n, h, w = pics.shape
    ref_slices = refs.shape[0] if ref_slices is None else ref_slices
    out = np.zeros((n, res_h, res_w))
    lib().eo_cross_corr_brute(_p(pics), _p(refs), _p(out), w, h, res_w, res_h, ref_slices,
                              n // ref_slices)
    return out


def cross_corr_fft(pic, ref):
    pic = np.ascontiguousarray(pic, dtype=np.float64)
    ref = np.ascontiguousarray(ref, dtype=np.float64)
    h2, w2 = pic.shape
    out = np.zeros((h2, w2))
    lib().eo_cross_corr_fft(_p(pic), _p(ref), w2, h2, _p(out))
    return out


def fft_c2c(x, inverse=False):
    d = np.ascontiguousarray(np.asarray(x, dtype=np.complex128)).copy()
    lib().eo_fft_c2c(d.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(d), int(inverse))
    return d


def maxarg(maps):
    maps = np.ascontiguousarray(maps, dtype=np.float64)
    n = maps.shape[0]
    size = maps[0].size
    idx = np.zeros(n, dtype=np.uint32)
    val = np.zeros(n)
    lib().eo_maxarg(_p(maps), size, n, _p(idx, ctypes.c_uint32), _p(val))
    return idx, val


def extract_neighbors(maps, idx, policy, cross_w, cross_h, s):
    maps = np.ascontiguousarray(maps, dtype=np.float64)
    idx = np.ascontiguousarray(idx, dtype=np.uint32)
    n = len(idx)
    out = np.zeros((n, s * s))
    lib().eo_extract_neighbors(_p(maps), _p(idx, ctypes.c_uint32), n, policy, cross_w,
                               cross_h, s, _p(out))
    return out


def subpixel_max(neigh, s):
    neigh = np.ascontiguousarray(neigh, dtype=np.float64).reshape(-1, s * s)
    n = neigh.shape[0]
    sub = np.zeros((n, 2))
    coefs = np.zeros((n, 6))
    if lib().eo_subpixel_max(_p(neigh), s, n, _p(sub), _p(coefs)) != 0:
        raise ValueError(f"unsupported fit size {s}")
    return sub, coefs


def shift_pos(index, policy, cross_w, cross_h):
    px, py = ctypes.c_uint32(), ctypes.c_uint32()
    lib().eo_shift_pos(ctypes.c_uint32(int(index)), policy, cross_w, cross_h,
                       ctypes.byref(px), ctypes.byref(py))
    return px.value, py.value


def get_offsets(ref_pattern, pics, begins, slice_w, slice_h, policy=POLICY_FFT,
                fitsize=3, cross_w=None, cross_h=None):
    """The whole path in FP64 (src/gpu_offset.hpp:127-301).

    ref_pattern: [H][W]; pics: [B][H][W]; both uint16 or float64.
    Returns (offsets [B*S][2], coefs [B*S][6], peaks [B*S]).
    """
    pics = np.ascontiguousarray(pics)
    if pics.ndim == 2:
        pics = pics[None]
    ref_pattern = np.ascontiguousarray(ref_pattern)
    in_type = IN_U16 if pics.dtype == np.uint16 else IN_F64
    if in_type == IN_F64:
        pics = pics.astype(np.float64)
        ref_pattern = ref_pattern.astype(np.float64)
    else:
        ref_pattern = ref_pattern.astype(np.uint16)
    b, h, w = pics.shape
    begins = np.ascontiguousarray(begins, dtype=np.uint32).reshape(-1, 2)
    n = b * len(begins)
    if cross_w is None:
        cross_w = 2 * slice_w - 1
    if cross_h is None:
        cross_h = 2 * slice_h - 1
    p = EoParams(w, h, _p(begins, ctypes.c_uint32), len(begins), slice_w, slice_h, cross_w,
                 cross_h, b, policy, fitsize, in_type)
    offs = np.zeros((n, 2))
    coefs = np.zeros((n, 6))
    peaks = np.zeros(n, dtype=np.uint32)
    rc = lib().eo_get_offsets(ctypes.byref(p), ref_pattern.ctypes.data_as(ctypes.c_void_p),
                              pics.ctypes.data_as(ctypes.c_void_p), _p(offs), _p(coefs),
                              _p(peaks, ctypes.c_uint32))
    if rc != 0:
        raise ValueError(f"oracle rejected the parameters (code {rc})")
    return offs, coefs, peaks


def homography_system(mids, offsets, centre):
    """The 2S x 9 homogeneous system of python/process_offsets.py:85-99 for one
    pattern: ROI centres (x, y) about the pattern centre, their offsets, and the
    centre's distance z; rows [-a z, -b z, -z^2, 0, 0, 0, a c, b c, z c] and
    [0, 0, 0, -a z, -b z, -z^2, a d, b d, z d] with c = a + dx, d = b + dy."""
    mids = np.asarray(mids, dtype=np.float64)
    offsets = np.asarray(offsets, dtype=np.float64)
    a = mids[:, 0] - centre[0]
    b = mids[:, 1] - centre[1]
    z = float(centre[2])
    c = a + offsets[:, 0]
    d = b + offsets[:, 1]
    A = np.zeros((2 * len(mids), 9))
    A[0::2, 0] = -a * z
    A[0::2, 1] = -b * z
    A[0::2, 2] = -z * z
    A[1::2, 3] = -a * z
    A[1::2, 4] = -b * z
    A[1::2, 5] = -z * z
    A[0::2, 6] = a * c
    A[0::2, 7] = b * c
    A[0::2, 8] = z * c
    A[1::2, 6] = a * d
    A[1::2, 7] = b * d
    A[1::2, 8] = z * d
    return A


def homography_fit(mids, offsets, centre):
    """python/process_offsets.py:83-104: the unit vector minimising |A x| (the
    right singular vector of the smallest singular value, from scipy's SVD as
    the reference calls it), as a 3x3 matrix divided by its [2, 2] entry."""
    from scipy.linalg import svd
    v = svd(homography_system(mids, offsets, centre))[2][8]
    uu = v.reshape((3, 3))
    return uu / uu[2, 2]
