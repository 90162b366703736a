"""emida_gb300: GB300-native (sm_103a) implementation of emida's EBSD ROI
cross-correlation path behind the reference's gpu_offset/get_offset interface.

The compute lives in libemida_gb.so (hand-written CUDA, C ABI in
include/emida_gb.h); this package is its Python host side.
"""
from ._lib import EmidaError, LIB_PATH  # noqa: F401
from .api import (  # noqa: F401
    CROSS_POLICY_BRUTE, CROSS_POLICY_FFT, DATA_INDEX_F32, DATA_INDEX_F64, DeviceBuffer,
    GpuOffset, MultiLayout, Server, device_count, fit_homography, get_offset, lstsq_matrix,
    pinned_array, read_results, subpixel_max,
)

__all__ = [
    "EmidaError", "GpuOffset", "MultiLayout", "Server", "get_offset", "DeviceBuffer", "device_count", "lstsq_matrix",
    "subpixel_max", "pinned_array", "fit_homography", "read_results", "CROSS_POLICY_BRUTE", "CROSS_POLICY_FFT", "DATA_INDEX_F32",
    "DATA_INDEX_F64",
    "LIB_PATH",
]
