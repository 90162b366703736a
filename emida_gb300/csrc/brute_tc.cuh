// brute_tc.cuh -- launcher interface of the tensor-core brute-force kernel
// (brute_tc.cu): the brute cross-correlation of src/cross_corr.cu:11-74 as a
// dense BF16 hi/lo contraction on tcgen05, fused with maxarg, neighbour
// extraction and the FP64 fit.
#pragma once

#include "common.cuh"

namespace emida_gb {

struct brute_tc_args {
    const uint16_t *pics;     // [n_patterns][src_h][src_w]
    uint32_t src_w, src_h;
    const uint2 *begins;      // [n_rois] ROI top-left (x, y)
    uint32_t n_rois, n_patterns;
    const double *ref_prep;   // [n_rois][64][64] prepared reference ROIs (FP64)
    const double *hann;       // [128]: x window then y window, FP64
    const double *lstsq;      // (A^T A)^-1 A^T, 6 x s*s
    int fitsize;
    double *offsets;          // [n_patterns * n_rois][2], pattern-major
    double *coefs;            // [..][6] or null
    void *maxes;              // data_index<float>[..] or null
    float *neigh;             // [..][s*s] or null
    uint32_t *err;            // device error word
};

// ROI side and lag window the kernel is built for.
constexpr uint32_t BRUTE_TC_SIDE = 64;
constexpr uint32_t BRUTE_TC_CROSS = 2 * BRUTE_TC_SIDE - 1;

// grid <= 0: one CTA per SM, less -grid CTAs.
cudaError_t launch_brute_tc(const brute_tc_args &a, int grid, cudaStream_t st);
// Dynamic shared memory of one CTA.
size_t brute_tc_smem_bytes();
// Loads the kernel without launching it (see preload_fused).
cudaError_t preload_brute_tc();

}  // namespace emida_gb
