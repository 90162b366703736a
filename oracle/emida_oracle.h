/*
 * emida_oracle.h -- CPU FP64 restatement of emida's ROI cross-correlation path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle: only tests/, the
 * smoke() entry point and bench.py's CPU-baseline / reference arm may load it.
 * The product (libemida_gb.so) never links or calls it.
 *
 * Parity is pinned against the reference's own golden vectors
 * (test/get_offset_test.cpp:10-27 and :120-200, test/cross_corr_test.cpp,
 * test/maxarg_test.cpp, test/subpixel_max_test.cpp, test/prepare_test.cpp,
 * test/sum_test.cpp) and, where the reference's sources are mounted, against the
 * reference's CPU code compiled by oracle/Makefile into oracle/_ref/.
 *
 * Layouts follow the reference (src/gpu_offset.hpp:41-45): patterns are
 * [batch][src_h][src_w] row-major, ROI results are pattern-major then
 * ROI-major (index = pattern * n_rois + roi), ROI positions are top-left
 * corners (x, y).
 */
#ifndef EMIDA_ORACLE_H
#define EMIDA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { EO_POLICY_BRUTE = 0, EO_POLICY_FFT = 1 };
enum { EO_IN_U16 = 0, EO_IN_F64 = 1 };

typedef struct eo_params {
    uint32_t src_w, src_h;        /* pattern size */
    const uint32_t *begins;       /* [n_rois][2] top-left (x, y) */
    uint32_t n_rois;
    uint32_t slice_w, slice_h;    /* ROI size */
    uint32_t cross_w, cross_h;    /* brute lag window (odd); FFT forces 2*slice-1 */
    uint32_t batch;               /* patterns per call */
    int32_t policy;               /* EO_POLICY_* */
    int32_t fitsize;              /* 3, 5, 7, 9 */
    int32_t in_type;              /* EO_IN_* */
} eo_params;

/* src/host_helpers.hpp:29-37: symmetric Hann window, n-1 denominator, FP64. */
void eo_hanning(size_t n, double *out);

/* src/sum.cu:109-158, test/sums_serial.hpp:7-32: per-ROI sums.  u16 input sums
 * wrap modulo 2^32 exactly like the reference's uint32 accumulator. */
void eo_roi_sums_u16(const uint16_t *pics, uint32_t src_w, uint32_t src_h,
                     const uint32_t *begins, uint32_t n_rois,
                     uint32_t slice_w, uint32_t slice_h, uint32_t batch,
                     uint32_t *sums);
void eo_roi_sums_f64(const double *pics, uint32_t src_w, uint32_t src_h,
                     const uint32_t *begins, uint32_t n_rois,
                     uint32_t slice_w, uint32_t slice_h, uint32_t batch,
                     double *sums);

/* src/prepare_pics.cu:11-42: out[roi][y*out_w + x] = (p - sum/area) * hx[x] * hy[y]
 * for x < slice_w, y < slice_h; other out elements are left untouched.
 * sums_f64 holds the per-ROI sums converted to double. */
void eo_prepare_f64(const void *pics, int32_t in_type, uint32_t src_w, uint32_t src_h,
                    const uint32_t *begins, uint32_t n_rois, uint32_t slice_w,
                    uint32_t slice_h, uint32_t out_w, uint32_t out_h, uint32_t batch,
                    const double *sums_f64, const double *hx, const double *hy,
                    double *out);
/* FP32 mirror of the same kernel for --precision float: the pixel is cast to
 * float, the sum is cast to float before the division (prepare_pics.cu:38). */
void eo_prepare_f32(const uint16_t *pics, uint32_t src_w, uint32_t src_h,
                    const uint32_t *begins, uint32_t n_rois, uint32_t slice_w,
                    uint32_t slice_h, uint32_t out_w, uint32_t out_h, uint32_t batch,
                    const uint32_t *sums, const float *hx, const float *hy, float *out);

/* src/cross_corr.cu:11-66: brute-force correlation
 * res[n][py][px] = sum_{y,x} pics[n][y+sy][x+sx] * ref[n % ref_slices][y][x],
 * (sx, sy) = (px, py) - (res - 1) / 2, over the overlap; y outer, x inner. */
void eo_cross_corr_brute(const double *pics, const double *ref, double *res,
                         uint32_t w, uint32_t h, uint32_t res_w, uint32_t res_h,
                         uint32_t ref_slices, uint32_t batch);

/* In-place complex FFT of length n (any n; mixed radix, prime lengths by
 * direct DFT).  data is interleaved (re, im).  inverse != 0: unnormalised
 * inverse (sign +1), which is what cuFFT's C2R/Z2D compute. */
void eo_fft_c2c(double *data, uint32_t n, int inverse);

/* FFT-policy correlation of one prepared pair (both [2h][2w] zero-padded real):
 * corr = C2R( R2C(pic) * conj(R2C(ref)) ), unnormalised
 * (src/gpu_offset.hpp:303-316, src/hadamard.cu:39-40).  out is [2h][2w]. */
void eo_cross_corr_fft(const double *pic, const double *ref, uint32_t w2, uint32_t h2,
                       double *out);

/* src/maxarg.cu: index of the maximum of each map, first occurrence in
 * row-major order wins ties. */
void eo_maxarg(const double *maps, uint32_t map_size, uint32_t n, uint32_t *idx,
               double *val);

/* src/extract_neighbors.cu:12-41 with the index policies of src/kernels.cuh:22-53.
 * cross_w/h is the lag-window size (127 for a 64 ROI).  Positions are clamped to
 * [0, cross] (inclusive, as the reference does); a flat index past the end of
 * the n-map buffer reads 0 (the reference reads past its allocation there). */
void eo_extract_neighbors(const double *maps, const uint32_t *idx, uint32_t n,
                          int32_t policy, uint32_t cross_w, uint32_t cross_h, int s,
                          double *neigh);

/* Exact (A^T A)^-1 A^T for the 6-term quadratic, A rows (1,x,y,x^2,xy,y^2),
 * x fastest (src/subpixel_max.hpp:42-67, python/A_gen.py:8-40), computed in
 * exact rational arithmetic and rounded once per entry.  out is [6][s*s].
 * Returns 0, or -1 for an unsupported s. */
int eo_lstsq_matrix(int s, double *out);

/* src/subpixel_max.hpp:76-97: coefficients (sequential FP64 dot products) and
 * the closed-form extremum.  sub is [n][2] (x, y), coefs [n][6]. */
int eo_subpixel_max(const double *neigh, int s, uint32_t n, double *sub, double *coefs);

/* src/kernels.cuh:30-33 / :47-52: argmax index -> lag-window position. */
void eo_shift_pos(uint32_t index, int32_t policy, uint32_t cross_w, uint32_t cross_h,
                  uint32_t *px, uint32_t *py);

/* The whole path: src/gpu_offset.hpp:127-301 (allocate_memory with the
 * reference pattern, get_offset_core, finalize).  offsets [batch*n_rois][2],
 * coefs [batch*n_rois][6] (may be NULL), peaks [batch*n_rois] (may be NULL).
 * Returns 0 or a negative error code. */
int eo_get_offsets(const eo_params *p, const void *ref_pattern, const void *pics,
                   double *offsets, double *coefs, uint32_t *peaks);

#ifdef __cplusplus
}
#endif
#endif
