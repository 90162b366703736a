// device_fit.cuh -- on-device neighbourhood extraction, FP64 quadratic fit and
// offset finalisation shared by the fused and the staged kernels.
//
// Mirrors src/extract_neighbors.cu:12-41 (index policies src/kernels.cuh:22-53),
// src/subpixel_max.hpp:76-97 and src/gpu_offset.hpp:289-298.  The fit uses
// explicitly rounded FP64 operations in the reference's order so that it gives
// the same bits as the host code built without FMA contraction.
#pragma once

#include "common.cuh"

namespace emida_gb {

// Lag-window position of an argmax index (src/kernels.cuh:30-33, :47-52).
__device__ __forceinline__ void shift_pos(uint32_t index, int policy, uint32_t cw, uint32_t ch,
                                          uint32_t &px, uint32_t &py)
{
    if (policy == POLICY_BRUTE) {
        px = index % cw;
        py = index / cw;
    } else {
        uint32_t iw = cw + 1, ih = ch + 1;
        px = (index % iw + (iw - 1) / 2) % iw;
        py = (index / iw + (ih - 1) / 2) % ih;
    }
}

// Index of lag-window position (x, y) inside one map (src/kernels.cuh:24-27, :39-45),
// relative to the map's own start.  For the brute policy the result can point
// past the map (the reference clamps to [0, cross] inclusive).
__device__ __forceinline__ uint64_t policy_index(int policy, uint32_t x, uint32_t y, uint32_t cw,
                                                 uint32_t ch)
{
    if (policy == POLICY_BRUTE) return (uint64_t)y * cw + x;
    uint32_t iw = cw + 1, ih = ch + 1;
    uint32_t ix = (x + (iw / 2 + 1)) % iw, iy = (y + (ih / 2 + 1)) % ih;
    return (uint64_t)iy * iw + ix;
}

// Clamped source position of neighbour (i, j) around the peak
// (src/extract_neighbors.cu:28-36).
__device__ __forceinline__ void neighbour_pos(uint32_t mx, uint32_t my, int i, int j, int s,
                                              uint32_t cw, uint32_t ch, uint32_t &x, uint32_t &y)
{
    int r = (s - 1) / 2;
    int fx = (int)mx - r + i, fy = (int)my - r + j;
    x = fx < 0 ? 0u : (uint32_t)fx;
    if (x > cw) x = cw;
    y = fy < 0 ? 0u : (uint32_t)fy;
    if (y > ch) y = ch;
}

// coef[c] = sum_k M[c][k] * v[k], sequential in k (src/subpixel_max.hpp:14-29).
// lstsq is (A^T A)^-1 A^T for this s, 6 rows of s*s, in global memory.
__device__ __forceinline__ double fit_coef(const double *__restrict__ lstsq, const double *v,
                                           int s, int c)
{
    const double *m = lstsq + c * s * s;
    double acc = 0.0;
    for (int k = 0; k < s * s; ++k) acc = __dadd_rn(acc, __dmul_rn(m[k], v[k]));
    return acc;
}

// Closed-form extremum (src/subpixel_max.hpp:91-92) and the offset
// (src/gpu_offset.hpp:296-297).
__device__ __forceinline__ void fit_offsets(const double *c, uint32_t mx, uint32_t my,
                                            uint32_t cw, uint32_t ch, int s, double &ox,
                                            double &oy)
{
    double b = c[1], cc = c[2], d = c[3], e = c[4], f = c[5];
    double num = __dsub_rn(__dmul_rn(b, e), __dmul_rn(__dmul_rn(2.0, cc), d));
    double den = __dsub_rn(__dmul_rn(__dmul_rn(4.0, f), d), __dmul_rn(e, e));
    double y = __ddiv_rn(num, den);
    double x = __ddiv_rn(__dsub_rn(__dmul_rn(-e, y), b), __dmul_rn(2.0, d));
    int r = (s - 1) / 2;
    ox = -__dadd_rn((double)((int)mx - (int)(cw / 2) - r), x);
    oy = -__dadd_rn((double)((int)my - (int)(ch / 2) - r), y);
}

}  // namespace emida_gb
