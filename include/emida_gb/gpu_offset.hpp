// gpu_offset.hpp -- C++ shim with the reference's driver interface over the
// C ABI of libemida_gb.so (include/emida_gb.h).
//
// A caller of the reference's  emida::gpu_offset<T, IN>  (src/gpu_offset.hpp:48-326)
// and  emida::get_offset  (src/get_offset.hpp:7-20) switches by including this
// header instead and linking libemida_gb.so: same namespace, class template,
// member signatures, types (src/common.hpp:24-145, src/subpixel_max.hpp:69-74)
// and failure behaviour (std::runtime_error).  The device buffers are freed by
// the destructor (the reference never frees them).
//
// The public in_stream and out_stream members are the library's own streams,
// set by allocate_memory; the caller's CUDA runtime accepts them
// (cudaStreamSynchronize(offs.in_stream) as src/process_files.hpp:196 does).
// This header needs no CUDA header: cudaStream_t is declared as the CUDA
// headers declare it, so either may be included first.
#pragma once

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../emida_gb.h"

struct CUstream_st;
typedef struct CUstream_st *cudaStream_t;

namespace emida {

using esize_t = uint32_t;

template <typename T>
struct vec2 {
    T x;
    T y;
    T area() const { return x * y; }
    vec2 operator+(const vec2 &r) const { return {x + r.x, y + r.y}; }
    vec2 operator-(const vec2 &r) const { return {x - r.x, y - r.y}; }
    template <typename U> vec2 operator*(const U &r) const { return {x * r, y * r}; }
    template <typename U> vec2 operator/(const U &r) const { return {x / r, y / r}; }
    template <typename U> vec2 operator-(const U &r) const { return {x - r, y - r}; }
    bool operator==(const vec2 &r) const { return x == r.x && y == r.y; }
};
using size2_t = vec2<esize_t>;

template <typename T>
struct data_index {
    T data;
    esize_t index;
};

enum cross_policy { CROSS_POLICY_BRUTE, CROSS_POLICY_FFT };

template <typename T>
struct offsets_t {
    std::vector<vec2<T>> offsets;
    std::vector<std::array<T, 6>> coefs;
};

inline void check_status(int status)
{
    if (status != EMIDA_GB_OK) throw std::runtime_error(emida_gb_last_error());
}

template <typename T, typename IN>
class gpu_offset {
    static_assert(std::is_same<T, float>::value || std::is_same<T, double>::value, "T: float or double");
    static_assert(std::is_same<IN, uint16_t>::value || std::is_same<IN, double>::value,
                  "IN: uint16_t or double");

    emida_gb_handle *h_ = nullptr;
    emida_gb_params p_{};
    std::vector<uint32_t> begins_;
    esize_t total_slices_ = 0;
    int s_ = 3;
    int mode_ = EMIDA_GB_MODE_AUTO;

public:
    // src/gpu_offset.hpp:96-97
    cudaStream_t in_stream = nullptr;
    cudaStream_t out_stream = nullptr;

    gpu_offset() {}
    gpu_offset(size2_t src_size, const std::vector<size2_t> *begins, size2_t slice_size,
               size2_t cross_size, esize_t batch_size, cross_policy policy = CROSS_POLICY_BRUTE,
               int s = 3, size_t in_buffers_size = 1, int mode = EMIDA_GB_MODE_AUTO)
        : total_slices_((esize_t)begins->size() * batch_size), s_(s), mode_(mode)
    {
        begins_.reserve(2 * begins->size());
        for (const auto &b : *begins) {
            begins_.push_back(b.x);
            begins_.push_back(b.y);
        }
        p_.src_w = src_size.x;
        p_.src_h = src_size.y;
        p_.n_rois = (uint32_t)begins->size();
        p_.slice_w = slice_size.x;
        p_.slice_h = slice_size.y;
        p_.cross_w = cross_size.x;
        p_.cross_h = cross_size.y;
        p_.batch_size = batch_size;
        p_.policy = policy == CROSS_POLICY_FFT ? EMIDA_GB_FFT : EMIDA_GB_BRUTE;
        p_.precision = std::is_same<T, double>::value ? EMIDA_GB_DOUBLE : EMIDA_GB_FLOAT;
        p_.fitsize = s;
        p_.in_type = std::is_same<IN, double>::value ? EMIDA_GB_IN_F64 : EMIDA_GB_IN_U16;
        p_.mode = mode;
        p_.in_buffers = (uint32_t)in_buffers_size;
    }
    gpu_offset(const gpu_offset &) = delete;
    gpu_offset &operator=(const gpu_offset &) = delete;
    gpu_offset(gpu_offset &&o) noexcept { *this = std::move(o); }
    gpu_offset &operator=(gpu_offset &&o) noexcept
    {
        std::swap(h_, o.h_);
        p_ = o.p_;
        begins_ = std::move(o.begins_);
        total_slices_ = o.total_slices_;
        s_ = o.s_;
        mode_ = o.mode_;
        std::swap(in_stream, o.in_stream);
        std::swap(out_stream, o.out_stream);
        return *this;
    }
    ~gpu_offset() { emida_gb_destroy(h_); }

    // src/gpu_offset.hpp:127-211
    void allocate_memory(IN *temp)
    {
        if (!h_) {
            p_.begins = begins_.data();
            check_status(emida_gb_create(&p_, &h_));
            void *in = nullptr, *out = nullptr;
            check_status(emida_gb_streams(h_, &in, &out));
            in_stream = static_cast<cudaStream_t>(in);
            out_stream = static_cast<cudaStream_t>(out);
        }
        if (temp) check_status(emida_gb_set_reference(h_, temp));
    }

    // src/gpu_offset.hpp:213-218
    esize_t transfer_pic_to_device_async(IN *pic)
    {
        uint32_t i = 0;
        check_status(emida_gb_transfer_async(h_, pic, &i));
        return i;
    }

    // src/gpu_offset.hpp:220-231 (the fit runs on the device)
    offsets_t<double> get_offset(IN *pic)
    {
        offsets_t<double> r;
        std::vector<double> o(2 * (size_t)total_slices_), c(6 * (size_t)total_slices_);
        check_status(emida_gb_get_offset(h_, pic, o.data(), c.data(), nullptr));
        unpack(o, c, r);
        return r;
    }

    // src/gpu_offset.hpp:234-278
    void get_offset_core(data_index<T> *maxes_i, T *neighbors, size_t cu_pic_index)
    {
        check_status(emida_gb_offsets_core(h_, (uint32_t)cu_pic_index, maxes_i, neighbors));
    }

    // src/gpu_offset.hpp:280-301
    offsets_t<double> finalize(data_index<T> *maxes_i, T *neighbors)
    {
        offsets_t<double> r;
        std::vector<double> o(2 * (size_t)total_slices_), c(6 * (size_t)total_slices_);
        check_status(emida_gb_finalize(h_, maxes_i, neighbors, o.data(), c.data()));
        unpack(o, c, r);
        return r;
    }

    // src/gpu_offset.hpp:303-316: R2C of get_cu_pic(), the conjugate product
    // with get_cu_temp()'s reference spectra, and the C2R into the correlation
    // maps (returns when they are done)
    void cross_corr_fft() const { check_status(emida_gb_cross_corr_fft(h_)); }

    // src/gpu_offset.hpp:318-321: device buffer of the prepared patterns
    T *get_cu_pic()
    {
        void *p = nullptr;
        check_status(emida_gb_stage_buffers(h_, &p, nullptr, nullptr));
        return static_cast<T *>(p);
    }
    // src/gpu_offset.hpp:322-325: device buffer of the reference spectra (FFT
    // policy) or of the prepared reference ROIs (brute policy)
    T *get_cu_temp()
    {
        void *p = nullptr;
        check_status(emida_gb_stage_buffers(h_, nullptr, &p, nullptr));
        return static_cast<T *>(p);
    }

    esize_t total_slices() const { return total_slices_; }
    emida_gb_handle *handle() { return h_; }

private:
    static void unpack(const std::vector<double> &o, const std::vector<double> &c, offsets_t<double> &r)
    {
        const size_t n = o.size() / 2;
        r.offsets.resize(n);
        r.coefs.resize(n);
        for (size_t i = 0; i < n; ++i) {
            r.offsets[i] = {o[2 * i], o[2 * i + 1]};
            for (int j = 0; j < 6; ++j) r.coefs[i][j] = c[6 * i + j];
        }
    }
};

// src/get_offset.hpp:7-14
template <typename T>
inline std::vector<vec2<T>> get_offset(T *pic, T *temp, size2_t size, size2_t cross_size,
                                       cross_policy c_policy = CROSS_POLICY_BRUTE)
{
    std::vector<size2_t> begins = {{0, 0}};
    gpu_offset<T, T> offs(size, &begins, size, cross_size, 1, c_policy);
    offs.allocate_memory(temp);
    auto o = offs.get_offset(pic).offsets;
    std::vector<vec2<T>> r(o.size());
    for (size_t i = 0; i < o.size(); ++i) r[i] = {(T)o[i].x, (T)o[i].y};
    return r;
}

// src/get_offset.hpp:16-20
template <typename T>
inline std::vector<vec2<T>> get_offset(T *pic, T *temp, size2_t size, size_t /*b_size*/)
{
    return get_offset(pic, temp, size, size2_t{2 * size.x - 1, 2 * size.y - 1});
}

}  // namespace emida
