// fused.cuh -- launcher interface of the fused FFT-policy kernel (fused.cu).
#pragma once

#include <cuda.h>

#include "common.cuh"

namespace emida_gb {

// How a uint16 ROI reaches shared memory.  TMA reads device memory only, so
// pinned host patterns (read in place over the host link) and pattern tables
// are staged by cp.async in 16-byte chunks, which also prefetches the next
// ROI behind the current one's column pass.
enum fused_stage : int {
    STAGE_PLAIN = 0,  // synchronous loads by every thread
    STAGE_TMA = 1,    // one TMA box per ROI (device-resident patterns), next ROI prefetched
    STAGE_ASYNC = 2,  // cp.async chunks of the ROI rows (src_w % 8 == 0, 16-byte aligned
                      // patterns; any memory the GPU can address), next ROI prefetched
};

struct fused_args {
    const void *pics;       // [batch][src_h][src_w] uint16 or double
    uint32_t src_w, src_h;
    const uint2 *begins;    // [n_rois] ROI top-left (x, y)
    uint32_t n_rois;
    uint32_t n_pairs;       // batch * n_rois
    uint32_t side;          // ROI side; <= N/2, zero-padded to N when smaller
    const void *ref_spec;   // [n_rois][N/2 + 1][N] complex: column kx holds X[0..N-1][kx]
    const void *hann;       // [2 * side]: x window then y window, element type T
    const void *twiddles;   // [N] complex T: exp(-2 pi i j / N)
    const double *lstsq;    // (A^T A)^-1 A^T, 6 x s*s
    int fitsize;
    int stage;              // fused_stage; TMA needs src_w % 8 == 0 and 16-byte aligned patterns
    double *offsets;        // [n_pairs][2]
    double *coefs;          // [n_pairs][6] or null
    void *maxes;            // data_index<T>[n_pairs] or null
    void *neigh;            // T[n_pairs][s*s] or null
    uint32_t *err;          // device error word (dev_err_t bits)
    // Work-list mode (several ROI layouts and fit sizes in one launch): item p
    // is {pattern, ROI index into begins / ref_spec, output slot, fit size}.
    // Without a list, pair p is pattern p / n_rois, ROI p % n_rois, slot p,
    // fit size `fitsize`.
    const uint4 *items;
    const double *lstsq_all; // items mode: the tables for s = 3, 5, 7, 9 back to back
    // Optional table of pattern base pointers: the pattern of item/pair p is
    // pattern_ptrs[pattern index] instead of pics + index * src_w * src_h.
    const void *const *pattern_ptrs;
    // ROI pairs per CTA: 0 for the length's default; the FP32 96-point kernel
    // with uint16 input takes 1, 2 or 4 (default: 2 with a pair queue, else 4)
    uint32_t pairs_per_cta;
    // Optional pair queue: two device words, zero at launch (the next round of
    // pairs past the first wave, the CTAs or clusters done).  CTA b starts on
    // round b (pairs b PPC .. b PPC + PPC - 1; cluster b of the 256-point
    // kernel on pair b) and takes each further round from the queue, so CTAs
    // on faster SMs take more pairs and the launch ends evenly; the last to
    // finish zeroes both words.  Launches that share a queue must be
    // stream-ordered.  Null: CTA b walks rounds b, b + grid, b + 2 grid, ...
    uint32_t *pair_queue;
};

// Offset of the s x s table inside lstsq_all (6*9, 6*25, 6*49, 6*81 doubles).
__host__ __device__ inline int lstsq_offset(int s)
{
    return s == 3 ? 0 : s == 5 ? 54 : s == 7 ? 204 : 498;
}

// Transform sizes with a fused kernel: 64, 96, 128 and, in FP32, 192 and 256
// (256 on a cluster of two CTAs, uint16 input only).
bool fused_supported(uint32_t fft_n, bool dbl, bool in_f64 = false);
// The smallest fused transform that holds a zero-padded ROI of this side (0: none).
uint32_t fused_size_for(uint32_t side, bool dbl, bool in_f64 = false);
// Loads the fused kernel of this length and types without launching it.  CUDA
// loads a kernel's module at its first use; done when a layout is registered,
// that cost (tens of milliseconds) stays out of the first request's latency.
cudaError_t preload_fused(uint32_t fft_n, bool dbl, bool in_f64);
// Dynamic shared memory of one CTA of the fused kernel for this length.
size_t fused_smem_bytes(uint32_t fft_n, bool dbl);
// Rows of the TMA box a CTA stages per ROI (the 256-point kernel's CTAs each
// stage half of the ROI).
uint32_t fused_box_rows(uint32_t fft_n, uint32_t side);

// grid <= 0: one wave of resident CTAs (occupancy x SM count) less -grid CTAs,
// which leaves room for a kernel that runs beside it (the gather of the next
// batch).
cudaError_t launch_fused(uint32_t fft_n, bool dbl, bool in_f64, const fused_args &a,
                         const CUtensorMap *tmap, int grid, cudaStream_t st);

}  // namespace emida_gb
