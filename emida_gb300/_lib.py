"""ctypes binding of libemida_gb.so (include/emida_gb.h).

The library is the product: there is no Python or CPU fallback.  Loading fails
loudly when the shared object is missing, and every call whose status is not
EMIDA_GB_OK raises EmidaError carrying emida_gb_last_error().
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libemida_gb.so")

OK = 0
BRUTE, FFT = 0, 1
DOUBLE, FLOAT = 0, 1
IN_U16, IN_F64 = 0, 1
MODE_AUTO, MODE_PLAIN, MODE_FUSED, MODE_TENSOR = 0, 1, 2, 3


class EmidaError(RuntimeError):
    """A failed C ABI call; the reference throws std::runtime_error there."""

    def __init__(self, status, message):
        super().__init__(f"emida_gb status {status}: {message}")
        self.status = status


class Params(ctypes.Structure):
    _fields_ = [
        ("src_w", ctypes.c_uint32), ("src_h", ctypes.c_uint32),
        ("begins", ctypes.POINTER(ctypes.c_uint32)), ("n_rois", ctypes.c_uint32),
        ("slice_w", ctypes.c_uint32), ("slice_h", ctypes.c_uint32),
        ("cross_w", ctypes.c_uint32), ("cross_h", ctypes.c_uint32),
        ("batch_size", ctypes.c_uint32), ("policy", ctypes.c_int32),
        ("precision", ctypes.c_int32), ("fitsize", ctypes.c_int32),
        ("in_type", ctypes.c_int32), ("mode", ctypes.c_int32),
        ("in_buffers", ctypes.c_uint32),
    ]


_lock = threading.Lock()
_lib = None

_VP = ctypes.c_void_p
_U32 = ctypes.c_uint32
_I32 = ctypes.c_int
_SZ = ctypes.c_size_t
_DP = ctypes.POINTER(ctypes.c_double)
_U32P = ctypes.POINTER(ctypes.c_uint32)

# name -> argument types (all return int unless listed in _RESTYPES)
SIGNATURES = {
    "emida_gb_create": [ctypes.POINTER(Params), ctypes.POINTER(_VP)],
    "emida_gb_set_reference": [_VP, _VP],
    "emida_gb_transfer_async": [_VP, _VP, _U32P],
    "emida_gb_offsets_core": [_VP, _U32, _VP, _VP],
    "emida_gb_finalize": [_VP, _VP, _VP, _DP, _DP],
    "emida_gb_get_offset": [_VP, _VP, _DP, _DP, _U32P],
    "emida_gb_submit": [_VP, _VP, _U32, ctypes.POINTER(ctypes.c_uint64)],
    "emida_gb_wait": [_VP, ctypes.c_uint64, _DP, _DP, _U32P],
    "emida_gb_run_device": [_VP, _VP, _U32, _VP, _VP, _VP, _VP, _VP],
    "emida_gb_multi_create": [_U32, _U32, _I32, ctypes.POINTER(_VP)],
    "emida_gb_multi_add_layout": [_VP, _U32P, _U32, _U32, _I32, _VP, _U32P],
    "emida_gb_multi_count": [_VP, _U32, _U32P, ctypes.POINTER(ctypes.c_uint64)],
    "emida_gb_multi_run": [_VP, _VP, _U32, _U32P, _VP, _VP, _VP, _I32],
    "emida_gb_multi_run_slots": [_VP, _VP, _U32, _U32, _U32P, _U32P, _VP, _VP, _VP],
    "emida_gb_multi_run_table": [_VP, ctypes.POINTER(_VP), _U32, _U32P, _VP, _VP, _VP],
    "emida_gb_multi_stream": [_VP],
    "emida_gb_multi_synchronize": [_VP],
    "emida_gb_multi_autotune": [_VP, _VP, _U32, _U32P, _VP, ctypes.c_char_p, _SZ],
    "emida_gb_multi_destroy": [_VP],
    "emida_gb_server_create": [_I32, ctypes.c_uint64, _U32, ctypes.POINTER(_VP)],
    "emida_gb_server_add_layout": [_VP, _U32, _U32, _U32P, _U32, _U32, _I32, _VP, _U32P],
    "emida_gb_server_submit": [_VP, _U32, _VP, _U32, ctypes.POINTER(ctypes.c_uint64)],
    "emida_gb_server_set_zero_copy": [_VP, _I32],
    "emida_gb_server_wait": [_VP, ctypes.c_uint64, _DP, _DP, _DP],
    "emida_gb_server_stats": [_VP, _DP, _DP, _DP, ctypes.POINTER(ctypes.c_uint64)],
    "emida_gb_server_reset_stats": [_VP],
    "emida_gb_server_trace": [_VP, _DP, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)],
    "emida_gb_server_destroy": [_VP],
    "emida_gb_resolved_mode": [_VP],
    "emida_gb_ingest": [_VP],
    "emida_gb_set_ingest": [_VP, _I32],
    "emida_gb_stream": [_VP],
    "emida_gb_streams": [_VP, ctypes.POINTER(_VP), ctypes.POINTER(_VP)],
    "emida_gb_stage_buffers": [_VP, ctypes.POINTER(_VP), ctypes.POINTER(_VP), ctypes.POINTER(_VP)],
    "emida_gb_cross_corr_fft": [_VP],
    "emida_gb_launches_per_run": [_VP],
    "emida_gb_destroy": [_VP],
    "emida_gb_last_error": [],
    "emida_gb_version": [],
    "emida_gb_subpixel_max": [_DP, _I32, _U32, _DP, _DP],
    "emida_gb_lstsq_matrix": [_I32, _DP],
    "emida_gb_device_count": [ctypes.POINTER(_I32)],
    "emida_gb_set_device": [_I32],
    "emida_gb_fit_homography": [_VP, _VP, _U32, _U32, _DP, _VP, ctypes.c_double, _VP, _VP],
    "emida_gb_time_fit_homography": [_VP, _VP, _U32, _U32, _DP, _VP, ctypes.c_double, _VP, _I32,
                                     ctypes.POINTER(ctypes.c_float)],
    "emida_gb_malloc": [ctypes.POINTER(_VP), _SZ],
    "emida_gb_free": [_VP],
    "emida_gb_memset": [_VP, _I32, _SZ],
    "emida_gb_memcpy_h2d": [_VP, _VP, _SZ],
    "emida_gb_memcpy_d2h": [_VP, _VP, _SZ],
    "emida_gb_memcpy_d2d": [_VP, _VP, _SZ],
    "emida_gb_malloc_host": [ctypes.POINTER(_VP), _SZ],
    "emida_gb_free_host": [_VP],
    "emida_gb_synchronize": [],
    "emida_gb_selftest_bounded_wait": [_VP, ctypes.c_int64],
    "emida_gb_selftest_arm_submit": [_VP, ctypes.c_int64],
    "emida_gb_time_device": [_VP, _VP, _U32, _VP, _I32, ctypes.POINTER(ctypes.c_float)],
    "emida_gb_run_sum": [_VP, _I32, _U32, _U32, _VP, _U32, _U32, _U32, _U32, _VP],
    "emida_gb_run_prepare": [_VP, _I32, _I32, _VP, _VP, _VP, _VP, _U32, _U32, _U32, _U32,
                             _U32, _U32, _U32, _U32],
    "emida_gb_run_cross_corr": [_VP, _VP, _VP, _I32, _U32, _U32, _U32, _U32, _U32, _U32],
    "emida_gb_run_fft_r2c": [_VP, _VP, _U32, _U32, _U32, _I32],
    "emida_gb_run_fft_r2c_noalloc": [_VP, _VP, _U32, _U32, _U32, _I32],
    "emida_gb_run_fft_c2r": [_VP, _VP, _U32, _U32, _U32, _I32],
    "emida_gb_run_hadamard": [_VP, _VP, _U32, _U32, _U32, _I32],
    "emida_gb_run_maxarg": [_VP, _U32, _U32, _VP, _I32],
    "emida_gb_run_extract_neighbors": [_VP, _VP, _VP, _I32, _U32, _U32, _U32, _I32, _I32],
}
_RESTYPES = {
    "emida_gb_last_error": ctypes.c_char_p,
    "emida_gb_version": ctypes.c_char_p,
    "emida_gb_stream": _VP,
    "emida_gb_multi_stream": _VP,
    "emida_gb_destroy": None,
    "emida_gb_multi_destroy": None,
    "emida_gb_server_destroy": None,
}


def lib():
    """The loaded library; raises if libemida_gb.so was not built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
                    "g.build()\"` (needs nvcc); there is no CPU fallback")
            L = ctypes.CDLL(LIB_PATH)
            for name, args in SIGNATURES.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = _RESTYPES.get(name, ctypes.c_int)
            _lib = L
    return _lib


def check(status):
    if status != OK:
        raise EmidaError(status, lib().emida_gb_last_error().decode(errors="replace"))
    return status


def call(name, *args):
    return check(getattr(lib(), name)(*args))
