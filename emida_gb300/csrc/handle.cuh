// handle.cuh -- the handle behind the C ABI and the host helpers shared by the
// translation units that drive it (capi.cu, multi.cu).
#pragma once

#include <cuda.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/emida_gb.h"
#include "common.cuh"
#include "brute_tc.cuh"
#include "fused.cuh"
#include "staged.cuh"

struct emida_gb_handle;

namespace emida_gb {
namespace host {

// An NVTX range over a scope, for timeline tools (nsys, ncu's range replay):
// the entry points of the C ABI and the request loop's stages are named after
// themselves.  Without a tool attached the calls do nothing.
struct trace_range {
    explicit trace_range(const char *name) { nvtxRangePushA(name); }
    ~trace_range() { nvtxRangePop(); }
    trace_range(const trace_range &) = delete;
    trace_range &operator=(const trace_range &) = delete;
};

// Records the message for emida_gb_last_error() and returns `code`.
int fail(int code, const char *fmt, ...);
// (A^T A)^-1 A^T for the 6-term quadratic, exact rationals rounded once.
int lstsq_matrix(int s, double *out);

using encode_fn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                               const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                               const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                               CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
encode_fn get_encoder();

int upload_hann(emida_gb_handle *h, void **dst, uint32_t nx, uint32_t ny);
int upload_twiddles(emida_gb_handle *h, void **dst, uint32_t n);
fft_tables tables(const emida_gb_handle *h);
// The staged pipeline for pats <= batch_size patterns (src/gpu_offset.hpp:234-278).
// With `ptrs` (device table) pattern p is ptrs[p]; with `out_base` (device,
// per pattern) its results land at output slots out_base[p] + roi, maxima in
// maxes_out.
int run_plain_chunk(emida_gb_handle *h, const void *pics, uint32_t pats, void *maxes, void *neigh,
                    double *offsets, double *coefs, cudaStream_t st,
                    const void *const *ptrs = nullptr, const uint32_t *out_base = nullptr,
                    void *maxes_out = nullptr);
// The pattern geometry a fused or tensor launch reads: the patterns as given,
// or the compact ROI layout that the gather ingest writes (patterns of
// gather_width(side) x n_rois * side pixels, ROI r at (x_r & 7, r * side)).
struct batch_view {
    size2 src;
    const uint2 *begins;
};
// `grid` as launch_fused and launch_brute_tc take it (<= 0: one wave less -grid CTAs);
// `err` the device error word the kernel sets (nullptr: the handle's).
int run_fused(emida_gb_handle *h, const void *pics, uint32_t pats, void *maxes, void *neigh,
              double *offsets, double *coefs, cudaStream_t st, const batch_view *view = nullptr,
              int grid = 0, uint32_t *err = nullptr);
int run_tensor(emida_gb_handle *h, const void *pics, uint32_t pats, void *maxes, void *neigh,
               double *offsets, double *coefs, cudaStream_t st, const batch_view *view = nullptr,
               int grid = 0, uint32_t *err = nullptr);
// Either form, any number of patterns (a view only for the fused and tensor forms).
int run_any(emida_gb_handle *h, const void *pics, uint32_t pats, void *maxes, void *neigh,
            double *offsets, double *coefs, cudaStream_t st, const batch_view *view = nullptr,
            int grid = 0, uint32_t *err = nullptr);
// Reads a device error word (nullptr: the handle's), clears it and reports its flags.
int check_device_error(emida_gb_handle *h, uint32_t *word = nullptr);
// EMIDA_GB_OK for no flags, else EMIDA_GB_DEVICE_CHECK with the flags named.
int device_flags_status(uint32_t flags);
// emida_gb_create with the fused transform length forced to fused_len (0: the
// smallest that holds the ROI), for the multi-layout autotuner.
int create_handle(const emida_gb_params *p, uint32_t fused_len, emida_gb_handle **out);
// CTA slots that a multi-layout planner's default one-wave launches leave free
// for kernels running beside them (0: none).
int multi_reserve_ctas(emida_gb_multi *m, int ctas);
// Sizes every work set of a multi-layout planner for runs of up to `patterns`
// patterns of its registered layouts, so that such runs allocate (and free,
// which waits for the whole device) nothing.
int multi_reserve_work(emida_gb_multi *m, uint32_t patterns);
// Recomputes the test hooks' reference spectra (fused and tensor forms) from
// the registered reference pattern; nothing when no hook buffers exist.
int stage_hooks_reference(emida_gb_handle *h);
// Host -> device copy of `patterns` whole patterns as the kernels need them:
// only the row bands that hold ROI pixels (one pitched copy per band over all
// patterns), or everything when the bands cover most of a pattern.
int copy_patterns(emida_gb_handle *h, void *dst, const void *src, uint32_t patterns, cudaStream_t st);
// Where a pattern array lives.  Device memory is staged through TMA; pinned
// host memory is read in place by the kernels (cp.async chunks over the
// NVLink-C2C host link on Grace systems), which skips the host-to-device copy
// of the pixels outside the ROIs.  Pageable memory is refused.
int pattern_location(const void *patterns, bool &on_device);

}  // namespace host
}  // namespace emida_gb

#define CK(expr)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (expr);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return emida_gb::host::fail(e_ == cudaErrorMemoryAllocation ? EMIDA_GB_OUT_OF_MEMORY             \
                                                        : EMIDA_GB_CUDA_ERROR,               \
                        "CUDA error %d (%s) at %s:%d: %s", (int)e_, cudaGetErrorString(e_),  \
                        __FILE__, __LINE__, #expr);                                         \
    } while (0)

#define CKS(expr)                                                                           \
    do {                                                                                    \
        int s_ = (expr);                                                                    \
        if (s_ != EMIDA_GB_OK) return s_;                                                   \
    } while (0)


using emida_gb::size2;
using emida_gb::data_index;

struct emida_gb_handle {
    emida_gb_params p{};
    std::vector<uint32_t> begins;
    int device = 0;
    bool dbl = false, in_f64 = false, fft = false;
    int mode = EMIDA_GB_MODE_PLAIN;
    size2 src{}, slice{}, cross{};
    uint32_t S = 0, B = 0, N = 0;
    uint32_t w2 = 0, h2 = 0, half = 0;
    size_t in_elem = 2, t_elem = 4, c_elem = 8, di_elem = 8;
    cudaStream_t in_stream = nullptr, out_stream = nullptr, comp = nullptr;
    std::vector<cudaEvent_t> in_done;
    std::vector<cudaEvent_t> in_used;  // per input buffer: offsets_core's kernels that read it
    cudaEvent_t comp_done = nullptr;
    cudaEvent_t out_done = nullptr;  // offsets_core's result copies on the output stream
    std::vector<void *> d_in;
    std::atomic<uint32_t> in_next{0};
    void *d_ref_in = nullptr;
    uint2 *d_begins = nullptr;
    void *d_hann = nullptr, *d_hann_fused = nullptr;
    double *d_hann64 = nullptr, *d_ref_prep64 = nullptr;  // tensor mode: FP64 reference ROIs
    void *d_sums_ref = nullptr, *d_sums = nullptr;
    void *d_ref_prep = nullptr, *d_prep = nullptr;
    void *d_ref_spec = nullptr, *d_ref_spec_cm = nullptr, *d_spec = nullptr;
    void *d_map = nullptr, *d_maxes = nullptr, *d_neigh = nullptr;
    double *d_offsets = nullptr, *d_coefs = nullptr, *d_lstsq = nullptr;
    void *d_tw_row = nullptr, *d_tw_col = nullptr;
    uint32_t *d_err = nullptr;
    // The fused kernel's pair queues (two words each, zero between launches):
    // one for launches on comp, one for comp_alt.  Launches on other streams
    // walk their pairs statically, as two of them could overlap on one queue.
    uint32_t *d_queues = nullptr;
    std::vector<double> lstsq;
    bool ref_set = false;
    // How submit brings pinned host batches to the kernels (EMIDA_GB_INGEST_*).
    // Reading in place is allowed when the ROIs cover at most half of each
    // pattern and a fused or tensor form runs.
    bool in_place_allowed = false;
    // rows [first, first + second) of a pattern that hold ROI pixels, merged
    std::vector<std::pair<uint32_t, uint32_t>> bands;
    int ingest = EMIDA_GB_INGEST_COPY;  // SM_COPY for the fused and tensor forms where allowed
    // The gather ingest: allowed for the fused and tensor forms with uint16
    // input, src_w % 8 == 0 and a compact layout no larger than the patterns;
    // d_begins_compact holds each ROI's place in the compact layout.
    bool gather_allowed = false;
    uint2 *d_begins_compact = nullptr;
    // The SM-copy ingest: the row bands as (first 16-byte chunk, chunks) runs
    // within a pattern; allowed when a pattern row is a whole number of
    // 16-byte chunks.
    bool sm_copy_allowed = false;
    uint2 *d_band_runs = nullptr;
    uint32_t n_band_runs = 0;
    std::mutex mu;
    std::vector<void *> allocs;
    // submit/wait ring: one slot per input buffer
    struct slot {
        double *d_offsets = nullptr, *d_coefs = nullptr;
        void *d_maxes = nullptr;
        double *h_offsets = nullptr, *h_coefs = nullptr;
        void *h_maxes = nullptr;
        uint32_t *d_err = nullptr;  // the error word this slot's path sets
        uint32_t *h_err = nullptr;  // its host copy, taken after the path
        cudaEvent_t h2d = nullptr, comp = nullptr, done = nullptr;
        uint64_t ticket = 0;
        uint32_t patterns = 0;
        bool busy = false;
    };
    std::vector<slot> ring;
    uint64_t next_ticket = 1;
    // Fused and tensor forms: batches of odd tickets run on this second compute
    // stream, so that a batch's path starts on the CTA slots the previous
    // batch's last CTAs leave free instead of after its tail.
    cudaStream_t comp_alt = nullptr;
    // The staged form's buffers behind emida_gb_stage_buffers and
    // emida_gb_cross_corr_fft (the reference's test hooks): the staged form's
    // own, or a set at the staged sizes made on first use by the other forms.
    struct stage_hook_buffers {
        bool ready = false;
        void *pic = nullptr, *temp = nullptr, *spec = nullptr, *map = nullptr, *ref_prep = nullptr;
        void *tw_row = nullptr, *tw_col = nullptr;
    } hk;
    // emida_gb_selftest_arm_submit: the next submit's slot word is set by a
    // bounded wait of this many cycles that runs out (0: not armed)
    int64_t selftest_budget = 0;

    int alloc(void **ptr, size_t bytes, bool zero = false)
    {
        if (bytes == 0) bytes = 16;
        CK(cudaMalloc(ptr, bytes));
        allocs.push_back(*ptr);
        if (zero) CK(cudaMemset(*ptr, 0, bytes));
        return EMIDA_GB_OK;
    }
    uint32_t map_size() const { return fft ? w2 * h2 : cross.x * cross.y; }
    size2 prep_size() const { return fft ? size2{w2, h2} : slice; }
};
