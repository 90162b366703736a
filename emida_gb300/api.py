"""Python mirror of the reference's driver interface over the C ABI.

`GpuOffset` follows `template<class T, class IN> class gpu_offset`
(src/gpu_offset.hpp:48-326) member by member; `get_offset` follows the free
function of src/get_offset.hpp:7-20.  Names, argument meaning and the
failure behaviour (an exception) are the reference's; the work is done by
libemida_gb.so.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import (BRUTE, DOUBLE, FFT, FLOAT, IN_F64, IN_U16, MODE_AUTO, MODE_FUSED, MODE_PLAIN,
                   MODE_TENSOR)

CROSS_POLICY_BRUTE, CROSS_POLICY_FFT = BRUTE, FFT

# data_index<T> of src/common.hpp:152-159 ({T data; uint32 index}, natural alignment)
DATA_INDEX_F32 = np.dtype([("data", "<f4"), ("index", "<u4")], align=True)
DATA_INDEX_F64 = np.dtype([("data", "<f8"), ("index", "<u4")], align=True)


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data)


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _precision(p):
    if p in (DOUBLE, "double", np.float64):
        return DOUBLE
    if p in (FLOAT, "float", np.float32):
        return FLOAT
    raise ValueError(f"Invalid precision argument: {p!r}")


def _policy(p):
    if p in (BRUTE, "brute"):
        return BRUTE
    if p in (FFT, "fft"):
        return FFT
    raise ValueError(f"Invalid crosspolicy argument: {p!r}")


def _mode(m):
    return {"auto": MODE_AUTO, "plain": MODE_PLAIN, "fused": MODE_FUSED, "tensor": MODE_TENSOR}.get(m, m)


class _PinnedBlock:
    """Pinned host memory from emida_gb_malloc_host, freed with its last user."""

    def __init__(self, nbytes):
        self.ptr = ctypes.c_void_p()
        _lib.call("emida_gb_malloc_host", ctypes.byref(self.ptr), max(1, int(nbytes)))

    def __del__(self):
        try:
            if self.ptr.value:
                _lib.lib().emida_gb_free_host(self.ptr)
                self.ptr = ctypes.c_void_p()
        except Exception:
            pass


def pinned_array(shape, dtype=np.uint16):
    """A numpy array in pinned (page-locked) host memory.  Pinned batches let
    copies overlap compute, and where a form reads its input in place (see
    GpuOffset.zero_copy) only the ROI pixels cross the host link."""
    dtype = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    block = _PinnedBlock(nbytes)
    buf = (ctypes.c_char * max(1, nbytes)).from_address(block.ptr.value)
    buf._block = block  # the memory lives as long as any view of it
    return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)


class DeviceBuffer:
    """A device allocation made through the C ABI (emida_gb_malloc)."""

    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        p = ctypes.c_void_p()
        _lib.call("emida_gb_malloc", ctypes.byref(p), self.nbytes)
        self.ptr = p

    @classmethod
    def from_array(cls, a):
        a = np.ascontiguousarray(a)
        b = cls(a.nbytes)
        b.upload(a)
        return b

    def upload(self, a):
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        _lib.call("emida_gb_memcpy_h2d", self.ptr, _ptr(a), a.nbytes)

    def download(self, dtype, shape):
        out = np.empty(shape, dtype=dtype)
        _lib.call("emida_gb_memcpy_d2h", _ptr(out), self.ptr, out.nbytes)
        return out

    def zero(self):
        _lib.call("emida_gb_memset", self.ptr, 0, self.nbytes)

    def free(self):
        if self.ptr is not None and self.ptr.value:
            _lib.lib().emida_gb_free(self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class GpuOffset:
    """gpu_offset<T, IN> (src/gpu_offset.hpp:48-326).

    src_size, slice_size, cross_size: (x, y) pairs; begins: ROI top-left (x, y)
    pairs; T is `precision` ("double" | "float"), IN is `in_dtype`
    (np.uint16 | np.float64).  `mode` selects the staged ("plain") or the fused
    form; "auto" takes the fused kernel where one covers the shape.
    """

    def __init__(self, src_size, begins, slice_size, cross_size, batch_size,
                 policy=CROSS_POLICY_BRUTE, s=3, in_buffers_size=1, precision="double",
                 in_dtype=np.uint16, mode="auto"):
        self.src_size = tuple(int(v) for v in src_size)
        self.begins = np.ascontiguousarray(np.asarray(begins, dtype=np.uint32).reshape(-1, 2))
        self.slice_size = tuple(int(v) for v in slice_size)
        self.policy = _policy(policy)
        if self.policy == FFT:
            cross_size = (2 * self.slice_size[0] - 1, 2 * self.slice_size[1] - 1)
        self.cross_size = tuple(int(v) for v in cross_size)
        self.batch_size = int(batch_size)
        self.s = int(s)
        self.precision = _precision(precision)
        self.T = np.float64 if self.precision == DOUBLE else np.float32
        self.in_dtype = np.dtype(in_dtype)
        if self.in_dtype not in (np.dtype(np.uint16), np.dtype(np.float64)):
            raise ValueError("IN must be uint16 or float64")
        self.total_slices = len(self.begins) * self.batch_size
        self.neigh_size = self.s * self.s * self.total_slices
        self.data_index = DATA_INDEX_F64 if self.precision == DOUBLE else DATA_INDEX_F32
        p = _lib.Params()
        p.src_w, p.src_h = self.src_size
        p.begins = self.begins.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
        p.n_rois = len(self.begins)
        p.slice_w, p.slice_h = self.slice_size
        p.cross_w, p.cross_h = self.cross_size
        p.batch_size = self.batch_size
        p.policy = self.policy
        p.precision = self.precision
        p.fitsize = self.s
        p.in_type = IN_U16 if self.in_dtype == np.dtype(np.uint16) else IN_F64
        p.mode = _mode(mode)
        p.in_buffers = int(in_buffers_size)
        h = ctypes.c_void_p()
        _lib.call("emida_gb_create", ctypes.byref(p), ctypes.byref(h))
        self._h = h
        self._pinned = []
        self._submitted = {}  # ticket -> patterns

    @property
    def handle(self):
        return self._h

    @property
    def mode(self):
        return {MODE_PLAIN: "plain", MODE_FUSED: "fused", MODE_TENSOR: "tensor"}[
            _lib.lib().emida_gb_resolved_mode(self._h)]

    def allocate_memory(self, temp=None):
        """src/gpu_offset.hpp:127-211: buffers exist from construction; with a
        reference pattern, prepares and transforms its ROIs once."""
        if temp is None:
            return
        temp = np.ascontiguousarray(temp, dtype=self.in_dtype)
        assert temp.size == self.src_size[0] * self.src_size[1]
        _lib.call("emida_gb_set_reference", self._h, _ptr(temp))

    def transfer_pic_to_device_async(self, pic):
        """src/gpu_offset.hpp:213-218.  Keeps `pic` alive until the next call on
        the same buffer; returns the buffer index."""
        pic = np.ascontiguousarray(pic, dtype=self.in_dtype)
        idx = ctypes.c_uint32()
        _lib.call("emida_gb_transfer_async", self._h, _ptr(pic), ctypes.byref(idx))
        self._pinned.append(pic)
        if len(self._pinned) > 64:
            self._pinned.pop(0)
        return idx.value

    def get_offset_core(self, cu_pic_index=0):
        """src/gpu_offset.hpp:234-278: returns (maxes_i, neighbors) host arrays,
        valid after finalize() (which waits for the output stream)."""
        maxes = np.zeros(self.total_slices, dtype=self.data_index)
        neigh = np.zeros(self.neigh_size, dtype=self.T)
        _lib.call("emida_gb_offsets_core", self._h, int(cu_pic_index), _ptr(maxes), _ptr(neigh))
        self._pinned.append((maxes, neigh))
        return maxes, neigh

    def finalize(self, maxes_i, neighbors):
        """src/gpu_offset.hpp:280-301: (offsets [n][2], coefs [n][6])."""
        offs = np.zeros((self.total_slices, 2))
        coefs = np.zeros((self.total_slices, 6))
        _lib.call("emida_gb_finalize", self._h, _ptr(maxes_i), _ptr(neighbors), _dptr(offs),
                  _dptr(coefs))
        return offs, coefs

    def get_offset(self, pic, with_peaks=False):
        """src/gpu_offset.hpp:220-231, with the fit on the device."""
        pic = np.ascontiguousarray(pic, dtype=self.in_dtype)
        assert pic.size == self.src_size[0] * self.src_size[1] * self.batch_size
        offs = np.zeros((self.total_slices, 2))
        coefs = np.zeros((self.total_slices, 6))
        peaks = np.zeros(self.total_slices, dtype=np.uint32)
        _lib.call("emida_gb_get_offset", self._h, _ptr(pic), _dptr(offs), _dptr(coefs),
                  peaks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
        if with_peaks:
            return offs, coefs, peaks
        return offs, coefs

    def submit(self, pic, patterns=None):
        """Queue one batch (host memory, pinned for overlap) and return a ticket.
        `pic` must stay alive and unchanged until wait(ticket).  An array
        batch holds len(pic) patterns unless `patterns` says fewer; an address
        holds batch_size patterns unless `patterns` says otherwise."""
        if isinstance(pic, int):
            patterns = self.batch_size if patterns is None else int(patterns)
            ptr = pic
        else:
            have = pic.size * pic.itemsize // (self.src_size[0] * self.src_size[1] * self.in_dtype.itemsize)
            patterns = have if patterns is None else int(patterns)
            if not pic.flags.c_contiguous or pic.dtype != self.in_dtype or patterns > have:
                raise ValueError(f"submit needs {patterns} contiguous {self.in_dtype} patterns")
            ptr = pic.ctypes.data
        t = ctypes.c_uint64()
        _lib.call("emida_gb_submit", self._h, ctypes.c_void_p(ptr), patterns, ctypes.byref(t))
        self._submitted[t.value] = patterns
        return t.value

    def wait(self, ticket, patterns=None, with_peaks=False):
        """Results of a submitted batch: (offsets, coefs[, peaks]), one row per
        ROI of each of its patterns."""
        if patterns is None:
            patterns = self._submitted.get(ticket, self.batch_size)
        n = int(patterns) * len(self.begins)
        offs = np.zeros((n, 2))
        coefs = np.zeros((n, 6))
        peaks = np.zeros(n, dtype=np.uint32)
        _lib.call("emida_gb_wait", self._h, ctypes.c_uint64(ticket), _dptr(offs), _dptr(coefs),
                  peaks.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
        self._submitted.pop(ticket, None)
        return (offs, coefs, peaks) if with_peaks else (offs, coefs)

    def run_device(self, dev_pics, patterns, dev_offsets, dev_coefs=None, dev_maxes=None,
                   dev_neigh=None, stream=None):
        """Device-resident form: any number of patterns, no synchronisation."""
        def vp(b):
            return None if b is None else (b.ptr if isinstance(b, DeviceBuffer) else ctypes.c_void_p(b))
        _lib.call("emida_gb_run_device", self._h, vp(dev_pics), int(patterns), vp(dev_offsets),
                  vp(dev_coefs), vp(dev_maxes), vp(dev_neigh),
                  None if stream is None else ctypes.c_void_p(stream))

    def time_device(self, dev_pics, patterns, dev_offsets, repeats):
        ms = ctypes.c_float()
        _lib.call("emida_gb_time_device", self._h, dev_pics.ptr, int(patterns), dev_offsets.ptr,
                  int(repeats), ctypes.byref(ms))
        return ms.value

    def stream(self):
        return _lib.lib().emida_gb_stream(self._h)

    # index = EMIDA_GB_INGEST_* value; 2 is not a mode
    INGEST = ("copy", "in_place", None, "gather", "sm_copy")

    @property
    def ingest(self):
        """How submit() brings pinned host batches to the kernels: "copy",
        "in_place" (kernels read the ROI pixels over the host link, no copy),
        "gather" (a gather kernel on a few SMs packs only the ROI rows into
        device memory beside the previous batch's path) or "sm_copy" (the
        row bands that "copy" moves, copied by SM loads on a few CTAs instead
        of the copy engine)."""
        return self.INGEST[_lib.lib().emida_gb_ingest(self._h)]

    @ingest.setter
    def ingest(self, mode):
        """In-place modes are honoured only when the ROIs cover at most half
        of each pattern (a fused or tensor form); "gather" only for a fused or
        tensor form with uint16 input, a width divisible by 8 and a compact
        ROI layout no larger than a pattern; "sm_copy" when a pattern row is
        a whole number of 16-byte chunks; otherwise "copy" stays."""
        if mode not in self.INGEST or mode is None:
            raise ValueError(f"unknown ingest mode {mode!r}")
        _lib.call("emida_gb_set_ingest", self._h, self.INGEST.index(mode))

    def launches_per_run(self):
        return _lib.lib().emida_gb_launches_per_run(self._h)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().emida_gb_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def get_offset(pic, temp, size, cross_size=None, c_policy=CROSS_POLICY_BRUTE, precision="double"):
    """src/get_offset.hpp:7-20: offsets of one ROI pair (the whole of `pic`
    against the whole of `temp`, both `size`), as gpu_offset<T, T> does."""
    pic = np.ascontiguousarray(pic, dtype=np.float64)
    temp = np.ascontiguousarray(temp, dtype=np.float64)
    size = tuple(int(v) for v in size)
    if cross_size is None:
        cross_size = (2 * size[0] - 1, 2 * size[1] - 1)
    g = GpuOffset(size, [(0, 0)], size, cross_size, 1, c_policy, 3, 1, precision, np.float64)
    try:
        g.allocate_memory(temp)
        offs, _ = g.get_offset(pic)
    finally:
        g.close()
    return offs


def lstsq_matrix(s):
    out = np.zeros(6 * s * s)
    _lib.call("emida_gb_lstsq_matrix", int(s), _dptr(out))
    return out.reshape(6, s * s)


def subpixel_max(neigh, s):
    """subpixel_max_serial (src/subpixel_max.hpp:76-97) on the host."""
    neigh = np.ascontiguousarray(neigh, dtype=np.float64).reshape(-1, s * s)
    sub = np.zeros((len(neigh), 2))
    coefs = np.zeros((len(neigh), 6))
    _lib.call("emida_gb_subpixel_max", _dptr(neigh), int(s), len(neigh), _dptr(sub), _dptr(coefs))
    return sub, coefs


def device_count():
    n = ctypes.c_int()
    st = _lib.lib().emida_gb_device_count(ctypes.byref(n))
    return n.value if st == 0 else 0


class MultiLayout:
    """Batches whose patterns use different ROI layouts (emida_gb_multi_*).

    add_layout() registers one layout (ROI top-left corners, ROI side, fit
    size) with its uint16 reference pattern and returns its id; run() processes
    device-resident uint16 patterns, pattern p with layout layout_of[p].  The
    results are flat in pattern order, then ROI order within the layout.
    """

    def __init__(self, src_size, precision="float"):
        self.src_size = tuple(int(v) for v in src_size)
        self.precision = _precision(precision)
        self.T = np.float64 if self.precision == DOUBLE else np.float32
        self.data_index = DATA_INDEX_F64 if self.precision == DOUBLE else DATA_INDEX_F32
        h = ctypes.c_void_p()
        _lib.call("emida_gb_multi_create", self.src_size[0], self.src_size[1], self.precision,
                  ctypes.byref(h))
        self._h = h
        self.layouts = []

    def add_layout(self, begins, side, fitsize, ref):
        begins = np.ascontiguousarray(np.asarray(begins, dtype=np.uint32).reshape(-1, 2))
        ref = np.ascontiguousarray(ref, dtype=np.uint16)
        lid = ctypes.c_uint32()
        _lib.call("emida_gb_multi_add_layout", self._h,
                  begins.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), len(begins), int(side),
                  int(fitsize), _ptr(ref), ctypes.byref(lid))
        self.layouts.append((begins, int(side), int(fitsize)))
        return lid.value

    def count(self, layout_of):
        lo = np.ascontiguousarray(layout_of, dtype=np.uint32)
        t = ctypes.c_uint64()
        _lib.call("emida_gb_multi_count", self._h, len(lo),
                  lo.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), ctypes.byref(t))
        return t.value

    def run(self, dev_pics, layout_of, dev_offsets, dev_coefs=None, dev_maxes=None, graph=True):
        self._lo = np.ascontiguousarray(layout_of, dtype=np.uint32)

        def vp(b):
            return None if b is None else b.ptr
        _lib.call("emida_gb_multi_run", self._h, vp(dev_pics), len(self._lo),
                  self._lo.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), vp(dev_offsets),
                  vp(dev_coefs), vp(dev_maxes), int(bool(graph)))

    def run_table(self, patterns, layout_of, dev_offsets, dev_coefs=None, dev_maxes=None):
        """One run over patterns given by address (device memory or pinned host
        memory read in place); `patterns` holds ints, DeviceBuffers or pinned
        arrays, which must stay alive until synchronize()."""
        self._lo = np.ascontiguousarray(layout_of, dtype=np.uint32)
        addr = [p.ptr.value if isinstance(p, DeviceBuffer) else
                (p.ctypes.data if isinstance(p, np.ndarray) else int(p)) for p in patterns]
        self._table = (ctypes.c_void_p * len(addr))(*addr)

        def vp(b):
            return None if b is None else b.ptr
        _lib.call("emida_gb_multi_run_table", self._h, self._table, len(addr),
                  self._lo.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), vp(dev_offsets),
                  vp(dev_coefs), vp(dev_maxes))

    def synchronize(self):
        _lib.call("emida_gb_multi_synchronize", self._h)

    def autotune(self, dev_pics, layout_of, dev_offsets):
        """emida_gb_multi_autotune: per ROI size class, times the candidate
        transform lengths, the tile shapes of each (ROI pairs per CTA) and
        grids of 1..6 CTAs per SM on these patterns, keeps the fastest, and
        returns the one-line-per-class report."""
        lo = np.ascontiguousarray(layout_of, dtype=np.uint32)
        buf = ctypes.create_string_buffer(4096)
        _lib.call("emida_gb_multi_autotune", self._h, dev_pics.ptr, len(lo),
                  lo.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), dev_offsets.ptr, buf, 4096)
        return buf.value.decode()

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().emida_gb_multi_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request loop over multi-layout batches (emida_gb_server_*).

    Rows of uint16 patterns are submitted against registered layouts; rows are
    admitted while the device arena of their pattern size has room (`hbm_bytes`
    per size) and computed in shared steps of up to `step_patterns` patterns.
    """

    def __init__(self, precision="float", hbm_bytes=8 << 30, step_patterns=64, zero_copy=False):
        self.precision = _precision(precision)
        h = ctypes.c_void_p()
        _lib.call("emida_gb_server_create", self.precision, int(hbm_bytes), int(step_patterns),
                  ctypes.byref(h))
        self._h = h
        self.rois = []
        self._rows = {}
        # True: every pinned row read in place; "sparse": rows of layouts whose
        # ROIs cover at most half of the pattern; False: every row copied into
        # the arena (by SM loads beside the running steps where aligned)
        level = 1 if zero_copy == "sparse" else 2 if zero_copy else 0
        _lib.call("emida_gb_server_set_zero_copy", h, level)

    def add_layout(self, src_size, begins, side, fitsize, ref):
        begins = np.ascontiguousarray(np.asarray(begins, dtype=np.uint32).reshape(-1, 2))
        ref = np.ascontiguousarray(ref, dtype=np.uint16)
        lid = ctypes.c_uint32()
        _lib.call("emida_gb_server_add_layout", self._h, int(src_size[0]), int(src_size[1]),
                  begins.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), len(begins), int(side),
                  int(fitsize), _ptr(ref), ctypes.byref(lid))
        self.rois.append(len(begins))
        return lid.value

    def submit(self, layout_id, patterns):
        """Queues a row; `patterns` ([n][h][w] uint16) is kept alive until wait()."""
        patterns = np.ascontiguousarray(patterns, dtype=np.uint16)
        rid = ctypes.c_uint64()
        _lib.call("emida_gb_server_submit", self._h, int(layout_id), _ptr(patterns), len(patterns),
                  ctypes.byref(rid))
        self._rows[rid.value] = (patterns, layout_id)
        return rid.value

    def wait(self, request_id):
        """(offsets [n*rois][2], coefs [n*rois][6], latency_ms) of a row."""
        patterns, lid = self._rows[request_id]
        n = len(patterns) * self.rois[lid]
        offs = np.zeros((n, 2))
        coefs = np.zeros((n, 6))
        lat = ctypes.c_double()
        try:
            _lib.call("emida_gb_server_wait", self._h, ctypes.c_uint64(request_id), _dptr(offs),
                      _dptr(coefs), ctypes.byref(lat))
        finally:
            del self._rows[request_id]
        return offs, coefs, lat.value

    def stats(self):
        p50, p99, rate = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        done = ctypes.c_uint64()
        _lib.call("emida_gb_server_stats", self._h, ctypes.byref(p50), ctypes.byref(p99),
                  ctypes.byref(rate), ctypes.byref(done))
        return {"p50_ms": p50.value, "p99_ms": p99.value, "pairs_per_s": rate.value,
                "completed": done.value}

    def trace(self):
        """Per completed row (completion order): [patterns, ms to admission,
        ms to its first step's launch, ms to its last step's launch, ms to
        completion], all from its submission."""
        n = ctypes.c_uint64()
        _lib.call("emida_gb_server_trace", self._h, None, 0, ctypes.byref(n))
        out = np.zeros((n.value, 5))
        if n.value:
            _lib.call("emida_gb_server_trace", self._h, _dptr(out), n.value, ctypes.byref(n))
        return out

    def reset_stats(self):
        _lib.call("emida_gb_server_reset_stats", self._h)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            _lib.lib().emida_gb_server_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fit_homography(mids, offsets, centre, coefs=None, min_det=1e-6):
    """The deformation fit after the path (python/process_offsets.py:83-104),
    batched on the GPU: per pattern, the 3x3 projective map carrying the ROI
    centres `mids` ([S][2], x, y) to their displaced positions, from the
    offsets ([P][S][2]) about `centre` = (cx, cy, z), divided by its [2][2]
    entry.  With `coefs` ([P][S][6] fit coefficients of the path), ROIs whose
    peak is not a clear maximum are left out as jove/analyze.py:44-56 does,
    and a pattern with ten or fewer kept ROIs gives NaN.  Returns [P][3][3]."""
    mids = np.ascontiguousarray(mids, dtype=np.float64).reshape(-1, 2)
    n = len(mids)
    offsets = np.ascontiguousarray(offsets, dtype=np.float64).reshape(-1, n, 2)
    p = len(offsets)
    d_mids, d_offs = DeviceBuffer.from_array(mids), DeviceBuffer.from_array(offsets)
    d_coefs = None
    if coefs is not None:
        d_coefs = DeviceBuffer.from_array(np.ascontiguousarray(coefs, dtype=np.float64).reshape(p, n, 6))
    d_out = DeviceBuffer(p * 9 * 8)
    c = (ctypes.c_double * 3)(*[float(v) for v in centre])
    _lib.call("emida_gb_fit_homography", d_mids.ptr, d_offs.ptr, n, p, c,
              d_coefs.ptr if d_coefs is not None else None, float(min_det), d_out.ptr, None)
    _lib.call("emida_gb_synchronize")
    return d_out.download(np.float64, (p, 3, 3))


def read_results(path):
    """Reads the CLI's --binary results file: a list of per-pattern dicts with
    x, y, name, mids [S][2] (uint32), offsets [S][2] and coefs [S][6]."""
    import struct
    out = []
    with open(path, "rb") as f:
        data = f.read()
    pos = 0
    rec = np.dtype([("mid", "<u4", 2), ("offset", "<f8", 2), ("coefs", "<f8", 6)])
    while pos < len(data):
        x, y, n, ln = struct.unpack_from("<ddII", data, pos)
        pos += 24
        name = data[pos:pos + ln].decode()
        pos += ln
        r = np.frombuffer(data, dtype=rec, count=n, offset=pos)
        pos += n * rec.itemsize
        out.append({"x": x, "y": y, "name": name, "mids": r["mid"].copy(),
                    "offsets": r["offset"].copy(), "coefs": r["coefs"].copy()})
    return out
