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
