// shim_driver.cpp -- a C++ caller of the reference's interface, compiled
// against include/emida_gb/gpu_offset.hpp by tests/test_shim.py.
//
//   shim_driver validate
//       a bad fit size must throw std::runtime_error (before any device work)
//   shim_driver run IN OUT
//       IN: u32 w, h, n_rois, batch, policy (0 brute, 1 fft), precision (0 double,
//           1 float), fitsize, mode; u32 begins[n_rois][2]; u16 reference[h][w];
//           u16 patterns[batch][h][w]
//       OUT: f64 offsets and coefs of get_offset, then of the pipeline
//            transfer_pic_to_device_async -> get_offset_core -> finalize
//   shim_driver pair IN OUT
//       IN: u32 size; f64 pic[size][size]; f64 temp[size][size]
//       OUT: f64 offset of the free function get_offset<double>(pic, temp, size, cross)
#include <cstdio>
#include <cstring>
#include <iostream>
#include <vector>

#include "emida_gb/gpu_offset.hpp"

namespace {

template <typename V> bool read_vec(FILE *f, std::vector<V> &v, size_t n)
{
    v.resize(n);
    return fread(v.data(), sizeof(V), n, f) == n;
}

template <typename T>
int run(uint32_t w, uint32_t h, const std::vector<emida::size2_t> &begins, uint32_t batch,
        emida::cross_policy policy, int s, int mode, std::vector<uint16_t> &ref,
        std::vector<uint16_t> &pics, FILE *out)
{
    const emida::size2_t src{w, h}, slice{64, 64}, cross{127, 127};
    emida::gpu_offset<T, uint16_t> offs(src, &begins, slice, cross, batch, policy, s, 1, mode);
    offs.allocate_memory(ref.data());
    auto one = offs.get_offset(pics.data());
    const size_t n = offs.total_slices();
    std::vector<emida::data_index<T>> maxes(n);
    std::vector<T> neigh(n * s * s);
    const auto buf = offs.transfer_pic_to_device_async(pics.data());
    offs.get_offset_core(maxes.data(), neigh.data(), buf);
    auto two = offs.finalize(maxes.data(), neigh.data());
    for (const auto *r : {&one, &two}) {
        for (size_t i = 0; i < n; ++i) fwrite(&r->offsets[i], sizeof(double), 2, out);
        for (size_t i = 0; i < n; ++i) fwrite(r->coefs[i].data(), sizeof(double), 6, out);
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    try {
        if (argc >= 2 && !strcmp(argv[1], "validate")) {
            std::vector<emida::size2_t> begins = {{0, 0}};
            emida::gpu_offset<double, uint16_t> offs({256, 256}, &begins, {64, 64}, {127, 127}, 1,
                                                     emida::CROSS_POLICY_FFT, /*s*/ 4);
            try {
                offs.allocate_memory(nullptr);
            } catch (const std::runtime_error &e) {
                std::cout << "runtime_error: " << e.what() << "\n";
                return 0;
            }
            std::cout << "no error\n";
            return 1;
        }
        if (argc == 4 && !strcmp(argv[1], "run")) {
            FILE *in = fopen(argv[2], "rb"), *out = fopen(argv[3], "wb");
            if (!in || !out) return 2;
            std::vector<uint32_t> hdr, raw;
            if (!read_vec(in, hdr, 8)) return 2;
            const uint32_t w = hdr[0], h = hdr[1], n_rois = hdr[2], batch = hdr[3];
            if (!read_vec(in, raw, 2 * (size_t)n_rois)) return 2;
            std::vector<emida::size2_t> begins(n_rois);
            for (uint32_t r = 0; r < n_rois; ++r) begins[r] = {raw[2 * r], raw[2 * r + 1]};
            std::vector<uint16_t> ref, pics;
            if (!read_vec(in, ref, (size_t)w * h) || !read_vec(in, pics, (size_t)batch * w * h)) return 2;
            const auto policy = hdr[4] ? emida::CROSS_POLICY_FFT : emida::CROSS_POLICY_BRUTE;
            const int rc = hdr[5] ? run<float>(w, h, begins, batch, policy, (int)hdr[6], (int)hdr[7], ref, pics, out)
                                  : run<double>(w, h, begins, batch, policy, (int)hdr[6], (int)hdr[7], ref, pics, out);
            fclose(in);
            fclose(out);
            return rc;
        }
        if (argc == 4 && !strcmp(argv[1], "pair")) {
            FILE *in = fopen(argv[2], "rb"), *out = fopen(argv[3], "wb");
            if (!in || !out) return 2;
            std::vector<uint32_t> hdr;
            std::vector<double> pic, temp;
            if (!read_vec(in, hdr, 1)) return 2;
            const uint32_t n = hdr[0];
            if (!read_vec(in, pic, (size_t)n * n) || !read_vec(in, temp, (size_t)n * n)) return 2;
            auto o = emida::get_offset<double>(pic.data(), temp.data(), {n, n}, {2 * n - 1, 2 * n - 1});
            fwrite(&o[0], sizeof(double), 2, out);
            fclose(in);
            fclose(out);
            return 0;
        }
    } catch (const std::exception &e) {
        std::cerr << "Error: " << e.what() << "\n";
        return 1;
    }
    std::cerr << "usage: shim_driver validate | run IN OUT | pair IN OUT\n";
    return 2;
}
