// deformation.cuh -- per-pattern projective fit from ROI offsets (deformation.cu).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace emida_gb {

// ROIs per pattern the fit takes: the 2S x 9 system lives in one CTA's shared memory.
constexpr uint32_t HOMOGRAPHY_MAX_ROIS = 1600;
constexpr uint32_t HOMOGRAPHY_MIN_ROIS = 5;

// mids [n_rois][2] ROI centres (x, y); offsets [patterns][n_rois][2]; coefs
// [patterns][n_rois][6] or null (no mask); out [patterns][9] row-major 3x3.
cudaError_t launch_homography(const double *mids, const double *offsets, uint32_t n_rois,
                              uint32_t patterns, double cx, double cy, double cz, const double *coefs,
                              double min_det, double *out, cudaStream_t st);

}  // namespace emida_gb
