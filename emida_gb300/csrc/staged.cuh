// staged.cuh -- launchers of the plain staged pipeline (staged.cu).
//
// One launcher per stage of the reference's get_offset_core
// (src/gpu_offset.hpp:234-278, launchers declared in src/kernels.cuh:56-125).
// All pointers are device pointers; every launch goes to the given stream.
#pragma once

#include "common.cuh"

namespace emida_gb {

enum in_type_t : int32_t { IN_U16 = 0, IN_F64 = 1 };

// src/sum.cu:109-167: sums[pair] over the ROI, pair = pattern * n_rois + roi.
// u16 input sums into uint32 (wrapping like the reference), f64 into double.
// With `ptrs` (a device table of pattern addresses), pattern p is ptrs[p]
// instead of pics + p * src.x * src.y.
cudaError_t run_sums(const void *pics, int in_type, size2 src, const uint2 *begins,
                     uint32_t n_rois, size2 slice, uint32_t batch, void *sums, cudaStream_t st,
                     const void *const *ptrs = nullptr);

// src/prepare_pics.cu:11-63: out[pair][y*out.x + x] = (p - sum/area) * hx[x] * hy[y].
// hann holds slice.x x-window values followed by slice.y y-window values.
cudaError_t run_prepare(const void *pics, int in_type, bool dbl, void *out, const void *hann,
                        const void *sums, const uint2 *begins, size2 src, size2 slice,
                        size2 out_size, uint32_t n_rois, uint32_t batch, cudaStream_t st,
                        const void *const *ptrs = nullptr);

// src/cross_corr.cu:11-74: brute-force lags, y-outer / x-inner sums with
// separately rounded products and sums (same bits as the FP64 oracle).
cudaError_t run_cross_corr(const void *pics, const void *ref, void *res, bool dbl, size2 size,
                           size2 res_size, uint32_t ref_slices, uint32_t batch, cudaStream_t st);

// Generic mixed-radix FFT lines (replaces the cuFFT plans of
// src/gpu_offset.hpp:171-183).  Spectra use cuFFT's R2C layout
// [maps][h2][w2/2 + 1].
struct fft_tables {
    const void *tw_row;  // exp(-2 pi i j / w2), j < w2, complex T
    const void *tw_col;  // exp(-2 pi i j / h2), j < h2, complex T
    uint32_t w2, h2;
};
cudaError_t run_fft_r2c(const void *real_in, void *spec, uint32_t maps, const fft_tables &t,
                        bool dbl, cudaStream_t st);
cudaError_t run_fft_c2r(void *spec, void *real_out, uint32_t maps, const fft_tables &t, bool dbl,
                        cudaStream_t st);

// src/hadamard.cu:26-49: pics[i] <- pics[i] * conj(ref[i mod (one_area * ref_slices)]).
cudaError_t run_hadamard(void *pics, const void *ref, uint32_t one_area, uint32_t ref_slices,
                         uint32_t batch, bool dbl, cudaStream_t st);

// src/maxarg.cu:180-187: per-map (max, index), first maximum in row-major order.
cudaError_t run_maxarg(const void *maps, uint32_t map_size, uint32_t n, void *maxes, bool dbl,
                       cudaStream_t st);

// src/extract_neighbors.cu:43-49 with the index policies of src/kernels.cuh:22-53.
cudaError_t run_extract_neighbors(const void *maps, const void *maxes, void *neigh, int s,
                                  size2 cross, uint32_t n, int policy, bool dbl, cudaStream_t st);

// On-device FP64 fit and finalisation (src/subpixel_max.hpp:76-97,
// src/gpu_offset.hpp:289-298).  coefs may be null.  With `out_base` (device,
// one entry per pattern of n_rois pairs) pair i lands in output slot
// out_base[i / n_rois] + i % n_rois, and its maximum is copied to
// maxes_out[slot] when maxes_out is given.
cudaError_t run_fit(const void *neigh, const void *maxes, uint32_t n, int s, size2 cross,
                    int policy, const double *lstsq, bool dbl, double *offsets, double *coefs,
                    cudaStream_t st, const uint32_t *out_base = nullptr, uint32_t n_rois = 1,
                    void *maxes_out = nullptr);

// Compact ROI layout for a batch that crosses the host link: row y of ROI r of
// pattern p lands at out + ((p * n_rois + r) * slice.y + y) * cw, cw =
// gather_width(slice.x) pixels from source pixel (x_r & ~7), so the ROI
// starts at column x_r & 7 of its compact rows.  Only the 16-byte chunks that
// hold ROI pixels are read; pics may be pinned host memory (read over
// NVLink-C2C) or device memory.  Needs src.x % 8 == 0 and 16-byte aligned
// pics and out; `ctas` bounds the grid (256 threads each).  Each CTA reserves
// `smem` bytes of (unused) dynamic shared memory: given the footprint of the
// kernel it runs beside, a gather CTA takes exactly one of that kernel's CTA
// slots, so the two fill one wave together whichever is dispatched first.
uint32_t gather_width(uint32_t side);
cudaError_t run_gather_rois(const uint16_t *pics, size2 src, const uint2 *begins, uint32_t n_rois,
                            size2 slice, uint32_t patterns, uint16_t *out, int ctas, size_t smem,
                            cudaStream_t st);

// Copy of the ROI row bands of `patterns` patterns from src (pinned host
// memory, read over NVLink-C2C) to dst in the same layout, by SM loads on at
// most `ctas` CTAs rather than by the copy engine.  runs[n_runs] holds each
// band as (first 16-byte chunk, chunk count) within a pattern of pat16
// chunks; src and dst 16-byte aligned.  Each CTA reserves `smem` bytes of
// (unused) dynamic shared memory, as run_gather_rois does.
cudaError_t run_copy_bands(const void *src, void *dst, const uint2 *runs, uint32_t n_runs,
                           uint64_t pat16, uint32_t patterns, int ctas, size_t smem,
                           cudaStream_t st);

// Reference spectra from cuFFT layout [S][h2][w2/2+1] to the fused kernel's
// column-major layout [S][w2/2+1][h2].
// Column 0 of each column-major n x (n/2 + 1) reference spectrum, replaced by
// the prepared reference ROI's row sums and alternating row sums (the inputs
// of the fused kernel's direct DC/Nyquist correlation); prep is [maps][n][n].
cudaError_t run_ref_row_sums(const void *prep, void *spec_cm, uint32_t maps, uint32_t n, bool dbl,
                             cudaStream_t st);
cudaError_t run_spec_to_colmajor(const void *spec, void *out, uint32_t maps, uint32_t w2,
                                 uint32_t h2, bool dbl, cudaStream_t st);

}  // namespace emida_gb
