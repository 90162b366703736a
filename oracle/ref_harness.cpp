// ref_harness.cpp -- extern "C" shims over the reference's own CPU code, compiled
// from the reference sources where they lie (see oracle/Makefile, target `ref`).
// TEST INFRASTRUCTURE ONLY: it exists to pin the oracle against the reference
// itself and, where it was built, to time the reference's CPU arithmetic.
// Nothing here is part of the product.
#include <cstdint>
#include <cstring>
#include <vector>

#include "cross_corr.hpp"    // src/cross_corr.hpp:29-65  cross_corr_serial
#include "subpixel_max.hpp"  // src/subpixel_max.hpp:14-97 subpixel_max_serial, lstsq tables
#include "subtract_mean.hpp" // src/subtract_mean.hpp:6-22
#include "host_helpers.hpp"  // src/host_helpers.hpp:29-37 generate_hanning
#include "sums_serial.hpp"   // test/sums_serial.hpp:7-32

using namespace emida;

namespace {

// One pattern's ROIs through the brute path on the CPU with the reference's
// own CPU code: sums_serial (test/sums_serial.hpp:7-32), generate_hanning
// (src/host_helpers.hpp:29-37), cross_corr_serial (src/cross_corr.hpp:29-65)
// and subpixel_max_serial (src/subpixel_max.hpp:76-97), in T.  The steps that
// the reference has only as GPU kernels are restated here: the mean
// subtraction and window of src/prepare_pics.cu:34-41, the first-maximum
// argmax of src/maxarg.cu, the s x s window of src/extract_neighbors.cu:20-39
// and the offset of src/gpu_offset.hpp:289-298.  offsets [n_rois][2],
// peaks [n_rois] (argmax index in the cross_w x cross_h map).
template <typename T>
void brute_offsets(const uint16_t *pattern, const T *ref_prepared, uint32_t w, uint32_t h,
                   const uint32_t *begins, uint32_t n_rois, uint32_t slice, uint32_t cross, int s,
                   double *offsets, uint32_t *peaks)
{
    const size2_t src{w, h}, ss{slice, slice}, cs{cross, cross};
    std::vector<size2_t> b(n_rois);
    for (uint32_t i = 0; i < n_rois; ++i) b[i] = size2_t{begins[2 * i], begins[2 * i + 1]};
    std::vector<uint16_t> pat(pattern, pattern + (size_t)w * h);
    const auto sums = sums_serial(pat, b, src, ss, 1);
    const auto hann = generate_hanning<T>(slice);
    const uint32_t area = slice * slice;
    std::vector<T> pic(area);
    std::vector<T> neigh((size_t)s * s);
    const int r = (s - 1) / 2;
    for (uint32_t i = 0; i < n_rois; ++i) {
        for (uint32_t y = 0; y < slice; ++y)
            for (uint32_t x = 0; x < slice; ++x) {
                T px = (T)pat[(size_t)(b[i].y + y) * w + b[i].x + x];
                px -= (T)sums[i] / area;
                pic[y * slice + x] = px * hann[x] * hann[y];
            }
        const auto res = cross_corr_serial<T>(pic.data(), ref_prepared + (size_t)i * area, ss, cs, 1);
        uint32_t best = 0;
        for (uint32_t k = 1; k < cs.area(); ++k)
            if (res[k] > res[best]) best = k;
        const int mx = (int)(best % cross), my = (int)(best / cross);
        for (int dy = 0; dy < s; ++dy)
            for (int dx = 0; dx < s; ++dx) {
                int x = mx - r + dx, y = my - r + dy;
                x = x < 0 ? 0 : (x > (int)cross ? (int)cross : x);
                y = y < 0 ? 0 : (y > (int)cross ? (int)cross : y);
                const size_t at = (size_t)y * cross + x;
                neigh[dy * s + dx] = at < res.size() ? res[at] : (T)0;
            }
        const auto sub = subpixel_max_serial<T>(neigh.data(), s, 1);
        offsets[2 * i] = -(mx - ((int)cross / 2) - r + sub.offsets[0].x);
        offsets[2 * i + 1] = -(my - ((int)cross / 2) - r + sub.offsets[0].y);
        if (peaks) peaks[i] = best;
    }
}

// The reference ROIs of one layout, prepared as above (src/gpu_offset.hpp:185-199
// does this for the reference pattern): [n_rois][slice][slice] T.
template <typename T>
void prepare_reference(const uint16_t *ref, uint32_t w, uint32_t h, const uint32_t *begins,
                       uint32_t n_rois, uint32_t slice, T *out)
{
    std::vector<size2_t> b(n_rois);
    for (uint32_t i = 0; i < n_rois; ++i) b[i] = size2_t{begins[2 * i], begins[2 * i + 1]};
    std::vector<uint16_t> pat(ref, ref + (size_t)w * h);
    const auto sums = sums_serial(pat, b, size2_t{w, h}, size2_t{slice, slice}, 1);
    const auto hann = generate_hanning<T>(slice);
    const uint32_t area = slice * slice;
    for (uint32_t i = 0; i < n_rois; ++i)
        for (uint32_t y = 0; y < slice; ++y)
            for (uint32_t x = 0; x < slice; ++x) {
                T px = (T)pat[(size_t)(b[i].y + y) * w + b[i].x + x];
                px -= (T)sums[i] / area;
                out[(size_t)i * area + y * slice + x] = px * hann[x] * hann[y];
            }
}

}  // namespace

extern "C" {

void ref_cross_corr_serial(const double* pics, const double* refs, uint32_t w, uint32_t h,
                           uint32_t res_w, uint32_t res_h, uint32_t ref_slices, double* out)
{
    auto res = cross_corr_serial<double>(pics, refs, size2_t{w, h}, size2_t{res_w, res_h},
                                         ref_slices);
    std::memcpy(out, res.data(), res.size() * sizeof(double));
}

int ref_lstsq_matrix(int s, double* out)
{
    try {
        const double* m = get_lstsq_matrix(s);
        std::memcpy(out, m, sizeof(double) * 6 * s * s);
        return 0;
    } catch (...) {
        return -1;
    }
}

void ref_subpixel_max_serial(const double* neigh, int s, uint32_t n, double* sub, double* coefs)
{
    auto r = subpixel_max_serial<double>(neigh, s, n);
    for (uint32_t i = 0; i < n; ++i) {
        sub[2 * i] = r.offsets[i].x;
        sub[2 * i + 1] = r.offsets[i].y;
        for (int j = 0; j < 6; ++j) coefs[6 * i + j] = r.coefs[i][j];
    }
}

void ref_subpixel_max_serial_f32(const float* neigh, int s, uint32_t n, double* sub, double* coefs)
{
    auto r = subpixel_max_serial<float>(neigh, s, n);
    for (uint32_t i = 0; i < n; ++i) {
        sub[2 * i] = r.offsets[i].x;
        sub[2 * i + 1] = r.offsets[i].y;
        for (int j = 0; j < 6; ++j) coefs[6 * i + j] = r.coefs[i][j];
    }
}

void ref_hanning(uint32_t n, double* out)
{
    auto v = generate_hanning<double>(n);
    std::memcpy(out, v.data(), n * sizeof(double));
}

void ref_subtract_mean(double* pic, uint32_t one_size, uint32_t b_size)
{
    subtract_mean(pic, one_size, b_size);
}

void ref_prepare_reference_f32(const uint16_t *ref, uint32_t w, uint32_t h, const uint32_t *begins,
                               uint32_t n_rois, uint32_t slice, float *out)
{
    prepare_reference<float>(ref, w, h, begins, n_rois, slice, out);
}
void ref_prepare_reference_f64(const uint16_t *ref, uint32_t w, uint32_t h, const uint32_t *begins,
                               uint32_t n_rois, uint32_t slice, double *out)
{
    prepare_reference<double>(ref, w, h, begins, n_rois, slice, out);
}
void ref_brute_offsets_f32(const uint16_t *pattern, const float *ref_prepared, uint32_t w, uint32_t h,
                           const uint32_t *begins, uint32_t n_rois, uint32_t slice, uint32_t cross,
                           int s, double *offsets, uint32_t *peaks)
{
    brute_offsets<float>(pattern, ref_prepared, w, h, begins, n_rois, slice, cross, s, offsets, peaks);
}
void ref_brute_offsets_f64(const uint16_t *pattern, const double *ref_prepared, uint32_t w, uint32_t h,
                           const uint32_t *begins, uint32_t n_rois, uint32_t slice, uint32_t cross,
                           int s, double *offsets, uint32_t *peaks)
{
    brute_offsets<double>(pattern, ref_prepared, w, h, begins, n_rois, slice, cross, s, offsets, peaks);
}

void ref_sums_serial(const double* data, uint32_t data_len, const uint32_t* begins, uint32_t n_begins,
                     uint32_t src_w, uint32_t src_h, uint32_t sw, uint32_t sh, uint32_t batch,
                     double* out)
{
    std::vector<double> d(data, data + data_len);
    std::vector<size2_t> b(n_begins);
    for (uint32_t i = 0; i < n_begins; ++i) b[i] = size2_t{begins[2 * i], begins[2 * i + 1]};
    auto r = sums_serial(d, b, size2_t{src_w, src_h}, size2_t{sw, sh}, batch);
    std::memcpy(out, r.data(), r.size() * sizeof(double));
}

}
