/*
 * emida_gb.h -- C ABI of the GB300-native emida ROI cross-correlation path.
 *
 * The entry points replace, one for one, the members of the reference's
 * driver class  template<class T, class IN> class gpu_offset
 * (src/gpu_offset.hpp:48-326) and its kernel launchers (src/kernels.cuh:56-125).
 * All functions return EMIDA_GB_OK (0) or a negative status; the message of the
 * last failure on the calling thread is returned by emida_gb_last_error().
 * The reference throws std::runtime_error instead (src/host_helpers.hpp:14-25);
 * the C++ shim include/emida_gb/gpu_offset.hpp turns statuses back into throws.
 *
 * Layouts (src/gpu_offset.hpp:41-45): a batch is [batch][src_h][src_w]
 * row-major pixels; results are pattern-major then ROI-major
 * (i = pattern * n_rois + roi).  Offsets are (x, y) doubles, coefficients the
 * six (a, b, c, d, e, f) of a + bx + cy + dx^2 + exy + fy^2.
 */
#ifndef EMIDA_GB_H
#define EMIDA_GB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    EMIDA_GB_OK = 0,
    EMIDA_GB_INVALID_ARGUMENT = -1,
    EMIDA_GB_CUDA_ERROR = -2,
    EMIDA_GB_UNSUPPORTED = -3,
    EMIDA_GB_DEVICE_CHECK = -4,
    EMIDA_GB_OUT_OF_MEMORY = -5
};

/* src/common.hpp:269-273 cross_policy */
enum { EMIDA_GB_BRUTE = 0, EMIDA_GB_FFT = 1 };
/* src/args_parser.hpp:14-18 precision_type (value order of this ABI) */
enum { EMIDA_GB_DOUBLE = 0, EMIDA_GB_FLOAT = 1 };
/* the IN template parameter of gpu_offset<T, IN> */
enum { EMIDA_GB_IN_U16 = 0, EMIDA_GB_IN_F64 = 1 };
/* execution form: AUTO picks FUSED where a fused kernel covers the shape.
 * TENSOR (requested explicitly, never chosen by AUTO): the brute policy on the
 * tcgen05 tensor cores with BF16 hi/lo split operands and FP32 accumulation,
 * fused with maxarg, neighbours and the FP64 fit; FLOAT precision, uint16
 * input, 64 x 64 ROIs and the full 127 x 127 lag window only.  Its offsets
 * agree with the FP64 path to about 1e-2 px instead of the FP32 paths' 1e-3. */
enum {
    EMIDA_GB_MODE_AUTO = 0,
    EMIDA_GB_MODE_PLAIN = 1,
    EMIDA_GB_MODE_FUSED = 2,
    EMIDA_GB_MODE_TENSOR = 3
};

typedef struct emida_gb_handle emida_gb_handle;

/* Constructor arguments of gpu_offset (src/gpu_offset.hpp:100-125). */
typedef struct emida_gb_params {
    uint32_t src_w, src_h;     /* pattern size (src_size) */
    const uint32_t *begins;    /* [n_rois][2] ROI top-left (x, y); copied */
    uint32_t n_rois;
    uint32_t slice_w, slice_h; /* ROI size (slice_size) */
    uint32_t cross_w, cross_h; /* brute lag window (odd); FFT forces 2*slice-1 */
    uint32_t batch_size;       /* patterns per batch */
    int32_t policy;            /* EMIDA_GB_BRUTE | EMIDA_GB_FFT */
    int32_t precision;         /* EMIDA_GB_DOUBLE | EMIDA_GB_FLOAT (the T parameter) */
    int32_t fitsize;           /* s = 3, 5, 7, 9 */
    int32_t in_type;           /* EMIDA_GB_IN_U16 | EMIDA_GB_IN_F64 (the IN parameter) */
    int32_t mode;              /* EMIDA_GB_MODE_* */
    uint32_t in_buffers;       /* device input buffers (in_buffers_size) */
} emida_gb_params;

/* gpu_offset ctor + the allocating half of allocate_memory
 * (src/gpu_offset.hpp:100-183).  Creates the streams and every device buffer. */
int emida_gb_create(const emida_gb_params *p, emida_gb_handle **out);

/* Reference half of allocate_memory (src/gpu_offset.hpp:185-210): sums,
 * prepare and forward FFT of the reference ROIs, kept resident.
 * ref: host pointer to one pattern of in_type pixels. */
int emida_gb_set_reference(emida_gb_handle *h, const void *ref);

/* transfer_pic_to_device_async (src/gpu_offset.hpp:213-218): asynchronous copy
 * of one batch from (pinned) host memory into the next input buffer on the
 * input stream; thread-safe; returns the buffer index.  The copy waits on the
 * device for the last emida_gb_offsets_core that read that buffer, as
 * offsets_core returns before its kernels have run. */
int emida_gb_transfer_async(emida_gb_handle *h, const void *batch, uint32_t *buffer_index);

/* get_offset_core (src/gpu_offset.hpp:234-278): runs the path on input buffer
 * `buffer_index` (after the input stream) and copies the per-ROI maxima
 * (data_index<T> {T value; uint32 index}) and s*s neighbourhoods (T) to the
 * host buffers, asynchronously on the output stream.  Either may be NULL.
 * Its kernels wait for the previous call's result copies, which read the
 * device buffers this call overwrites. */
int emida_gb_offsets_core(emida_gb_handle *h, uint32_t buffer_index, void *maxes_out,
                          void *neigh_out);

/* finalize (src/gpu_offset.hpp:280-301): waits for the output stream and fits
 * the neighbourhoods on the host.  offsets [n][2]; coefs [n][6] or NULL. */
int emida_gb_finalize(emida_gb_handle *h, const void *maxes, const void *neigh,
                      double *offsets, double *coefs);

/* get_offset (src/gpu_offset.hpp:220-231): synchronous copy of one batch,
 * the whole path on the device including the FP64 fit, and the results.
 * coefs and peaks (uint32 argmax index per ROI) may be NULL. */
int emida_gb_get_offset(emida_gb_handle *h, const void *batch, double *offsets, double *coefs,
                        uint32_t *peaks);

/* Pipelined form of get_offset for a stream of batches: queues the copy of
 * `patterns` (<= batch_size) patterns from host memory (pinned for overlap) on
 * the input stream, the path on the compute stream and the copy of the results
 * on the output stream, and returns a ticket at once.  Up to in_buffers batches
 * may be in flight; a ticket must be waited for before its slot is reused
 * (EMIDA_GB_INVALID_ARGUMENT otherwise).  The host batch must stay untouched
 * until its ticket is waited for.  The process_files pipeline of the reference
 * (src/process_files.hpp:98-233) does the same with threads and two streams.
 * A batch in device memory is used in place.  A batch in pinned host memory
 * arrives as emida_gb_set_ingest chose (default EMIDA_GB_INGEST_SM_COPY for
 * the fused and tensor forms where it is allowed, else EMIDA_GB_INGEST_COPY). */
int emida_gb_submit(emida_gb_handle *h, const void *batch, uint32_t patterns, uint64_t *ticket);
/* Waits for a ticket and copies its offsets [patterns*n_rois][2], coefficients
 * [..][6] and argmax indices [..] to the host (coefs, peaks may be NULL). */
int emida_gb_wait(emida_gb_handle *h, uint64_t ticket, double *offsets, double *coefs,
                  uint32_t *peaks);

/* Device-resident form for pipelines and benchmarks: `patterns` whole
 * patterns (any count, not limited to batch_size) already in device memory,
 * or in pinned host memory that the kernels read in place (only the 16-byte
 * chunks that hold ROI pixels cross the host link), results to device memory,
 * all on `stream`
 * (NULL: the handle's compute stream), no synchronisation.  Pageable host
 * memory is refused (EMIDA_GB_INVALID_ARGUMENT).  coefs, maxes, neigh may be
 * NULL.  On the handle's compute stream the fused kernels hand out their
 * pairs through a device queue (faster SMs take more); on another stream each
 * CTA walks a fixed set of pairs.  The results are the same bits. */
int emida_gb_run_device(emida_gb_handle *h, const void *dev_patterns, uint32_t patterns,
                        double *dev_offsets, double *dev_coefs, void *dev_maxes,
                        void *dev_neigh, void *stream);

/* Which form the handle runs: EMIDA_GB_MODE_PLAIN, _FUSED or _TENSOR. */
int emida_gb_resolved_mode(const emida_gb_handle *h);
/* How emida_gb_submit brings a pinned host batch to the kernels:
 *   COPY      a copy on the input stream, overlapping the previous batch's path;
 *   IN_PLACE  no copy: the kernels read the batch's ROI pixels in place over the
 *             host link (lowest latency per batch);
 *   GATHER    a gather kernel on a few SMs reads only the 16-byte chunks that
 *             hold ROI pixels over the host link into a compact device layout,
 *             beside the previous batch's path (the fewest bytes over the link
 *             and the lowest latency per batch; with several batches in flight
 *             the copy engine keeps up better, as the gather's host reads slow
 *             down beside the path's CTAs).
 *   SM_COPY   the ROI row bands, as COPY moves them, copied by SM loads on a
 *             few CTAs beside the previous batch's path rather than by the
 *             copy engine (a pitched copy engine transfer of the bands runs
 *             below the link's rate; SM loads of whole runs reach it).
 * Value 2 is not a mode (it named an alternating mode that was withdrawn, as it
 * was slower than every other); emida_gb_set_ingest refuses it.
 * IN_PLACE is taken only by a fused or tensor form whose ROIs cover
 * at most half of each pattern; GATHER by a fused or tensor form with uint16
 * input, src_w a multiple of 8 and a compact layout (n_rois ROIs of side x
 * ((side + 14) & ~7) pixels) no larger than a pattern, and only for 16-byte
 * aligned batches (others are copied); SM_COPY when a pattern row is a whole
 * number of 16-byte chunks, and only for 16-byte aligned batches (others are
 * copied).  Otherwise the mode stays COPY.
 * emida_gb_ingest reports the mode in force. */
enum {
    EMIDA_GB_INGEST_COPY = 0,
    EMIDA_GB_INGEST_IN_PLACE = 1,
    EMIDA_GB_INGEST_GATHER = 3,
    EMIDA_GB_INGEST_SM_COPY = 4
};
int emida_gb_set_ingest(emida_gb_handle *h, int mode);
int emida_gb_ingest(const emida_gb_handle *h);
/* The handle's compute stream (a cudaStream_t).  The fused kernels launched on
 * it share one pair queue, which stream order keeps to one launch at a time:
 * work captured from this stream into a graph must not run while other work
 * of the handle runs. */
void *emida_gb_stream(emida_gb_handle *h);
/* The public in_stream and out_stream members of gpu_offset
 * (src/gpu_offset.hpp:96-97): the streams of transfer_async's copies and of
 * offsets_core's result copies, as cudaStream_t values that the caller's own
 * CUDA runtime accepts (src/process_files.hpp:196 synchronises in_stream).
 * Either pointer may be NULL. */
int emida_gb_streams(emida_gb_handle *h, void **in_stream, void **out_stream);
/* The test hooks get_cu_pic() and get_cu_temp() of gpu_offset
 * (src/gpu_offset.hpp:318-325), plus the correlation maps they produce:
 * device buffers of the staged form, T = the handle's precision.
 *   FFT policy:   pic  [batch*n_rois][2*slice_h][2*slice_w] T, the prepared,
 *                      zero-padded ROIs (the R2C input);
 *                 temp [n_rois][2*slice_h][slice_w+1] complex T, the reference
 *                      spectra (computed by set_reference);
 *                 maps [batch*n_rois][2*slice_h][2*slice_w] T, the C2R output.
 *   brute policy: pic  [batch*n_rois][slice_h][slice_w] T, temp [n_rois][slice_h]
 *                 [slice_w] T (the prepared reference ROIs), maps
 *                 [batch*n_rois][cross_h][cross_w] T.
 * The staged form (EMIDA_GB_MODE_PLAIN) returns the buffers its
 * offsets_core uses; the fused and tensor forms keep no such buffers, so the
 * first call makes a set at these sizes for the hooks alone.  Any pointer may
 * be NULL. */
int emida_gb_stage_buffers(emida_gb_handle *h, void **pic, void **temp, void **maps);
/* The test hook cross_corr_fft() (src/gpu_offset.hpp:303-316): R2C of the
 * pic buffer, the product with the conjugate reference spectra of temp, and
 * the unnormalised C2R into maps, on the compute stream; returns when done.
 * FFT policy only. */
int emida_gb_cross_corr_fft(emida_gb_handle *h);
/* Number of kernel launches one emida_gb_run_device call makes. */
int emida_gb_launches_per_run(const emida_gb_handle *h);
void emida_gb_destroy(emida_gb_handle *h);

const char *emida_gb_last_error(void);
const char *emida_gb_version(void);

/* Host fit of s*s neighbourhoods (src/subpixel_max.hpp:76-97); values are
 * doubles.  sub [n][2] (x, y) inside the window, coefs [n][6] or NULL. */
int emida_gb_subpixel_max(const double *neigh, int s, uint32_t n, double *sub, double *coefs);
/* (A^T A)^-1 A^T used by the fit, 6 x s*s (src/subpixel_max.cpp:5-58). */
int emida_gb_lstsq_matrix(int s, double *out);

/* ---- multi-layout batches -------------------------------------------------
 * No counterpart in the reference, which runs one ROI layout per gpu_offset.
 * Patterns of one batch may each use a different layout (ROI positions, one
 * ROI side, one fit size), all against uint16 reference patterns.  Each
 * layout's reference spectra are computed once and stay resident.  A run
 * processes device-resident uint16 patterns with one persistent fused launch
 * per transform size (sizes without a fused kernel run the staged pipeline per
 * pattern).  Results are flat in pattern order, then ROI order within the
 * pattern's layout (emida_gb_multi_count gives the total). */
typedef struct emida_gb_multi emida_gb_multi;
int emida_gb_multi_create(uint32_t src_w, uint32_t src_h, int32_t precision,
                          emida_gb_multi **out);
int emida_gb_multi_add_layout(emida_gb_multi *m, const uint32_t *begins, uint32_t n_rois,
                              uint32_t side, int32_t fitsize, const uint16_t *ref,
                              uint32_t *layout_id);
int emida_gb_multi_count(const emida_gb_multi *m, uint32_t patterns, const uint32_t *layout_of,
                         uint64_t *total);
/* Queues a run on the planner's stream (no synchronisation).  use_graph != 0:
 * the launches are captured in a CUDA graph on first use and replayed while
 * the same patterns pointer, layout assignment and output pointers repeat.
 * dev_coefs [total][6] and dev_maxes (data_index<T>[total]) may be NULL. */
int emida_gb_multi_run(emida_gb_multi *m, const void *dev_patterns, uint32_t patterns,
                       const uint32_t *layout_of, double *dev_offsets, double *dev_coefs,
                       void *dev_maxes, int use_graph);
/* The same for patterns at arbitrary positions of a device pattern array of
 * `arena` patterns: entry p reads pattern slots[p]; no graph. */
int emida_gb_multi_run_slots(emida_gb_multi *m, const void *dev_patterns, uint32_t arena,
                             uint32_t patterns, const uint32_t *slots, const uint32_t *layout_of,
                             double *dev_offsets, double *dev_coefs, void *dev_maxes);
/* The same with one pointer per pattern: patterns[p] is pattern p in device
 * memory or in pinned host memory, which the kernels then read in place (only
 * the ROI pixels cross the host link).  The pointers and the memory behind
 * them must stay valid until the run has completed; no graph. */
int emida_gb_multi_run_table(emida_gb_multi *m, const void *const *patterns, uint32_t n,
                             const uint32_t *layout_of, double *dev_offsets, double *dev_coefs,
                             void *dev_maxes);
/* The planner's stream (a cudaStream_t) and a wait for its work.  Every run of
 * the planner launches on this stream, whose order keeps the fused kernels'
 * shared pair queue to one launch at a time. */
void *emida_gb_multi_stream(emida_gb_multi *m);
int emida_gb_multi_synchronize(emida_gb_multi *m);
/* Per ROI size class with a fused kernel, times on these patterns each
 * candidate transform length (the smallest that holds the ROI and the next
 * one, which zero-pads it further), each tile shape of that length's kernel
 * (ROI pairs per CTA: 4, 2 or 1 for the FP32 96-point kernel, 1 elsewhere),
 * with grids of 1..6 times the SM count (clusters of two CTAs at 256
 * points); keeps the fastest length, shape and grid, rebuilds the class's
 * resident reference spectra at that length, and writes a one-line-per-class
 * report. */
int emida_gb_multi_autotune(emida_gb_multi *m, const void *dev_patterns, uint32_t patterns,
                            const uint32_t *layout_of, double *dev_offsets, char *report,
                            size_t report_len);
void emida_gb_multi_destroy(emida_gb_multi *m);

/* ---- serving: a request loop over multi-layout batches ----------------------
 * No counterpart in the reference (its process_files pipeline runs one layout,
 * one row at a time).  A request is a scan row of n uint16 patterns on one
 * registered layout.  Rows wait until the device pattern arena of their size
 * (hbm_bytes per pattern size) can hold all their patterns, then are copied in
 * and computed in steps of up to step_patterns patterns drawn from every
 * admitted row in turn, so rows that arrive while others run share the next
 * steps.  The host patterns must stay valid until the request is waited for;
 * pinned memory lets the copies overlap.  A row's ROI row bands are copied in
 * chunks of 16 patterns, by SM loads on 16 CTAs beside the running steps when
 * the row is pinned and 16-byte aligned and a pattern row is a whole number of
 * 16-byte chunks (the steps leave those CTA slots free), else by the copy
 * engine.  emida_gb_server_set_zero_copy can instead have the kernels read
 * pinned rows' ROI pixels in place.  Results are per row, pattern-major. */
typedef struct emida_gb_server emida_gb_server;
int emida_gb_server_create(int32_t precision, uint64_t hbm_bytes, uint32_t step_patterns,
                           emida_gb_server **out);
int emida_gb_server_add_layout(emida_gb_server *s, uint32_t src_w, uint32_t src_h,
                               const uint32_t *begins, uint32_t n_rois, uint32_t side,
                               int32_t fitsize, const uint16_t *ref, uint32_t *layout_id);
int emida_gb_server_submit(emida_gb_server *s, uint32_t layout_id, const uint16_t *patterns,
                           uint32_t n, uint64_t *request_id);
/* Which pinned rows submitted later are read in place rather than copied into
 * the arena: 2 every pinned row, 1 rows of layouts whose ROIs cover at most
 * half of the pattern, 0 none (default).  A row read in place needs no arena
 * slots, but its steps run at the host link's rate for scattered ROI rows
 * (about 11 M ROI pairs/s at 1024^2 with 100 ROIs of 64^2); copied rows run
 * at the device-resident rate while the next rows' copies proceed beside them. */
int emida_gb_server_set_zero_copy(emida_gb_server *s, int enable);
/* Blocks until the row is done; offsets [n*rois][2], coefs [n*rois][6] may be
 * NULL; latency_ms = submission to completion. */
int emida_gb_server_wait(emida_gb_server *s, uint64_t request_id, double *offsets, double *coefs,
                         double *latency_ms);
/* p50/p99 row latency of completed rows and ROI pairs/s since the first submission. */
int emida_gb_server_stats(emida_gb_server *s, double *p50_ms, double *p99_ms,
                          double *pairs_per_s, uint64_t *completed);
/* Per-row timeline of the rows completed since the last reset, in completion
 * order: rows[i][0..4] = patterns, then ms from submission to admission, to
 * the launch of the row's first step, to the launch of its last step, and to
 * completion.  Writes min(count, capacity) rows (rows may be NULL to ask for
 * the count only). */
int emida_gb_server_trace(emida_gb_server *s, double *rows, uint64_t capacity, uint64_t *count);
int emida_gb_server_reset_stats(emida_gb_server *s);
void emida_gb_server_destroy(emida_gb_server *s);

/* ---- device memory helpers (for callers without a CUDA runtime binding) --- */
int emida_gb_device_count(int *count);

/* ---- the step after the path: deformation fit (python/process_offsets.py:83-104) ----
 * Per pattern, the projective map that carries the ROI centres to their
 * displaced positions, up to scale: the unit 9-vector minimising |A x| for the
 * 2S x 9 system built from centres (x, y) about centre = {cx, cy, z} and the
 * offsets, as a row-major 3x3 divided by its [2][2] entry.  mids [n_rois][2],
 * offsets [patterns][n_rois][2] and out [patterns][9] in device (or pinned host)
 * memory; 5 <= n_rois <= 1600.  coefs ([patterns][n_rois][6], the fit
 * coefficients of the path) may be NULL; when given, ROIs whose peak is not a
 * clear maximum (det of the negated quadratic <= min_det) are left out, and a
 * pattern with ten or fewer kept ROIs gives NaN (jove/analyze.py:44-56).
 * Queued on `stream` (NULL: the legacy stream), no synchronisation. */
int emida_gb_fit_homography(const double *mids, const double *offsets, uint32_t n_rois,
                            uint32_t patterns, const double *centre, const double *coefs,
                            double min_det, double *out, void *stream);
/* CUDA-event time of `repeats` fits (ms, all repeats together). */
int emida_gb_time_fit_homography(const double *mids, const double *offsets, uint32_t n_rois,
                                 uint32_t patterns, const double *centre, const double *coefs,
                                 double min_det, double *out, int repeats, float *ms);
/* Device for this thread's subsequent handles and helpers (one process per GPU). */
int emida_gb_set_device(int device);
int emida_gb_malloc(void **dev_ptr, size_t bytes);
int emida_gb_free(void *dev_ptr);
int emida_gb_memset(void *dev_ptr, int value, size_t bytes);
int emida_gb_memcpy_h2d(void *dev_dst, const void *host_src, size_t bytes);
int emida_gb_memcpy_d2h(void *host_dst, const void *dev_src, size_t bytes);
int emida_gb_memcpy_d2d(void *dev_dst, const void *dev_src, size_t bytes);
int emida_gb_malloc_host(void **host_ptr, size_t bytes);
int emida_gb_free_host(void *host_ptr);
int emida_gb_synchronize(void);
/* Self-test of the bounded waits every device spin loop uses: one warp waits
 * on an mbarrier phase that nothing completes, for about `budget_cycles` SM
 * clock cycles (at most 4e9, ~2 s).  The wait runs out, sets the handle's
 * device error word, and the call returns what a real timeout returns:
 * EMIDA_GB_DEVICE_CHECK, "pipeline wait ran out".  The context and the
 * handle stay usable; the error word is cleared.  No reference counterpart. */
int emida_gb_selftest_bounded_wait(emida_gb_handle *h, int64_t budget_cycles);
/* Self-test of a failed batch in the submit/wait ring: the next emida_gb_submit
 * on this handle sets its slot's device error word by the same bounded wait
 * (about budget_cycles cycles, at most 4e9) before the batch's path runs.  Its
 * emida_gb_wait then returns EMIDA_GB_DEVICE_CHECK ("pipeline wait ran out"),
 * consumes the ticket and frees the slot, and later batches run as usual.
 * One-shot; no fault, trap or hang.  No reference counterpart. */
int emida_gb_selftest_arm_submit(emida_gb_handle *h, int64_t budget_cycles);
/* CUDA-event timing on a stream: elapsed ms of `repeats` runs of the handle's
 * device form over the same inputs, measured on the launching stream. */
int emida_gb_time_device(emida_gb_handle *h, const void *dev_patterns, uint32_t patterns,
                         double *dev_offsets, int repeats, float *ms);

/* ---- per-stage launchers (src/kernels.cuh:56-125), device pointers -------- */
/* run_sum: sums[pair] over each ROI; u16 -> uint32, f64 -> double. */
int emida_gb_run_sum(const void *pics, int in_type, uint32_t src_w, uint32_t src_h,
                     const uint32_t *dev_begins, uint32_t n_rois, uint32_t slice_w,
                     uint32_t slice_h, uint32_t batch, void *sums);
/* run_prepare_pics: hann = slice_w x-window values then slice_h y-window values (T). */
int emida_gb_run_prepare(const void *pics, int in_type, int precision, void *slices,
                         const void *hann, const void *sums, const uint32_t *dev_begins,
                         uint32_t src_w, uint32_t src_h, uint32_t slice_w, uint32_t slice_h,
                         uint32_t out_w, uint32_t out_h, uint32_t n_rois, uint32_t batch);
/* run_cross_corr (brute): res [ref_slices*batch][res_h][res_w]. */
int emida_gb_run_cross_corr(const void *pics, const void *ref, void *res, int precision,
                            uint32_t w, uint32_t h, uint32_t res_w, uint32_t res_h,
                            uint32_t ref_slices, uint32_t batch);
/* forward R2C of [maps][h2][w2] real into [maps][h2][w2/2+1] complex (cuFFT layout). */
int emida_gb_run_fft_r2c(const void *real_in, void *spec, uint32_t maps, uint32_t w2,
                         uint32_t h2, int precision);
/* Allocation-free form of emida_gb_run_fft_r2c (no counterpart in the reference):
 * same arguments, same results, bit for bit.  It is for callers that must not
 * allocate device memory during a run: cudaFree synchronises the whole device,
 * which would stall a pipeline's other streams, and a caller whose memory pool
 * has claimed the free HBM up front has nothing left to allocate from.  Its
 * twiddle tables live in one fixed 32 KiB device array shared by every call,
 * so w2 and h2 must each be 1..1024 (larger sizes return
 * EMIDA_GB_INVALID_ARGUMENT), and calls that overlap in time on the same
 * device (from other host threads) race on that array.  The call runs on a
 * non-blocking stream of the library's own and waits for that stream only:
 * it orders nothing against the caller's streams, so real_in must be complete
 * before the call and spec is complete when it returns.  The first call on
 * each device, with that device current, looks the array's address up and
 * creates the stream; make that first call before any stream capture begins
 * (a condition on the first call only, not a statement about later calls).
 * Each call writes both tables before its kernels read them, so nothing in
 * the array has to start at zero. */
int emida_gb_run_fft_r2c_noalloc(const void *real_in, void *spec, uint32_t maps, uint32_t w2,
                                 uint32_t h2, int precision);
/* unnormalised C2R of [maps][h2][w2/2+1] (overwritten) into [maps][h2][w2] real. */
int emida_gb_run_fft_c2r(void *spec, void *real_out, uint32_t maps, uint32_t w2, uint32_t h2,
                         int precision);
/* run_hadamard: pics[i] *= conj(ref[i mod (one_area*ref_slices)]) (complex T). */
int emida_gb_run_hadamard(void *pics, const void *ref, uint32_t one_area, uint32_t ref_slices,
                          uint32_t batch, int precision);
/* run_maxarg_reduce: maxes[i] = {max, first index} of map i. */
int emida_gb_run_maxarg(const void *maps, uint32_t map_size, uint32_t n, void *maxes,
                        int precision);
/* run_extract_neighbors with the policy's index map. */
int emida_gb_run_extract_neighbors(const void *maps, const void *maxes, void *neigh, int s,
                                   uint32_t cross_w, uint32_t cross_h, uint32_t n, int policy,
                                   int precision);

#ifdef __cplusplus
}
#endif
#endif
