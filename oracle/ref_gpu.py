"""ctypes front end of the reference's own staged GPU pipeline
(oracle/_ref/libemida_ref_gpu.so, built by `make -C oracle ref_gpu` from the
sources staged into baseline/_ref; see oracle/ref_gpu_harness.cu).

TEST AND MEASUREMENT INFRASTRUCTURE ONLY: the reference's gpu_offset<T,
uint16_t> (src/gpu_offset.hpp:48-326) with cuFFT, used by tests/ as a second
FP64 check and by bench.py as the plain staged baseline.  Nothing in the
product imports it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libemida_ref_gpu.so")

_lib = None


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        if not available():
            raise ImportError(f"{LIB_PATH} is missing (make -C oracle stage ref_gpu REF=...)")
        L = ctypes.CDLL(LIB_PATH)
        vp, u32 = ctypes.c_void_p, ctypes.c_uint32
        dp = ctypes.POINTER(ctypes.c_double)
        L.refgpu_last_error.restype = ctypes.c_char_p
        L.refgpu_create.argtypes = [ctypes.c_int, u32, u32, ctypes.POINTER(u32), u32, u32, u32, u32,
                                    ctypes.c_int, ctypes.c_int, u32, vp, ctypes.POINTER(vp)]
        L.refgpu_get_offset.argtypes = [vp, vp, dp, dp]
        L.refgpu_run_batch.argtypes = [vp, vp, dp, dp, ctypes.POINTER(u32)]
        L.refgpu_time_core.argtypes = [vp, ctypes.POINTER(vp), u32, ctypes.c_int, dp]
        L.refgpu_time_e2e.argtypes = [vp, ctypes.POINTER(vp), u32, dp, dp]
        L.refgpu_destroy.argtypes = [vp]
        L.refgpu_destroy.restype = None
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        raise RuntimeError("reference gpu_offset: " + lib().refgpu_last_error().decode(errors="replace"))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class RefGpuOffset:
    """gpu_offset<T, uint16_t> of the reference: precision "float" | "double",
    policy "fft" | "brute", square ROIs of side `slice`, lag window `cross`
    (the FFT policy forces 2 slice - 1).  Pattern buffers passed to run_batch
    and the timers must be pinned host memory, as the reference's pipeline
    uses (src/process_files.hpp:102-104)."""

    def __init__(self, ref, begins, slice_, batch, policy="fft", s=5, precision="float",
                 cross=None, in_buffers=1):
        ref = np.ascontiguousarray(ref, dtype=np.uint16)
        h, w = ref.shape
        self.begins = np.ascontiguousarray(np.asarray(begins, dtype=np.uint32).reshape(-1, 2))
        self.n = len(self.begins) * int(batch)
        self.batch = int(batch)
        self.shape = (h, w)
        cross = cross or 2 * slice_ - 1
        self._h = ctypes.c_void_p()
        _check(lib().refgpu_create(0 if precision == "double" else 1, w, h,
                                   self.begins.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                   len(self.begins), slice_, cross, self.batch,
                                   1 if policy == "fft" else 0, s, in_buffers,
                                   ref.ctypes.data_as(ctypes.c_void_p), ctypes.byref(self._h)))

    def get_offset(self, batch):
        """The reference's get_offset (src/gpu_offset.hpp:220-231): (offsets, coefs)."""
        batch = np.ascontiguousarray(batch, dtype=np.uint16)
        assert batch.size == self.batch * self.shape[0] * self.shape[1]
        offs, coefs = np.zeros((self.n, 2)), np.zeros((self.n, 6))
        _check(lib().refgpu_get_offset(self._h, batch.ctypes.data_as(ctypes.c_void_p), _dp(offs), _dp(coefs)))
        return offs, coefs

    def run_batch(self, pinned_batch):
        """transfer_pic_to_device_async, cudaStreamSynchronize(in_stream),
        get_offset_core, finalize: (offsets, coefs, peaks)."""
        offs, coefs = np.zeros((self.n, 2)), np.zeros((self.n, 6))
        peaks = np.zeros(self.n, dtype=np.uint32)
        _check(lib().refgpu_run_batch(self._h, ctypes.c_void_p(pinned_batch.ctypes.data), _dp(offs),
                                      _dp(coefs), peaks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))))
        return offs, coefs, peaks

    @staticmethod
    def _table(batches):
        return (ctypes.c_void_p * len(batches))(*[b.ctypes.data for b in batches])

    def time_core(self, pinned_batches, repeats):
        """Host ms of `repeats` passes of get_offset_core over the batches, which
        sit in the input buffers (one buffer per batch: in_buffers >= len)."""
        ms = ctypes.c_double()
        _check(lib().refgpu_time_core(self._h, self._table(pinned_batches), len(pinned_batches),
                                      int(repeats), ctypes.byref(ms)))
        return ms.value

    def time_e2e(self, pinned_batches):
        """Host ms of the batches through transfer, get_offset_core and finalize."""
        ms = ctypes.c_double()
        scratch = np.zeros((self.n, 2))
        _check(lib().refgpu_time_e2e(self._h, self._table(pinned_batches), len(pinned_batches),
                                     _dp(scratch), ctypes.byref(ms)))
        return ms.value

    def close(self):
        if self._h is not None and self._h.value:
            lib().refgpu_destroy(self._h)
        self._h = None
