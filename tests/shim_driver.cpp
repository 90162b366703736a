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
//   shim_driver files IN OUT
//       IN: as `run`, then u32 n_patterns, load_workers; u32 begins[n_rois][2];
//           u16 reference[h][w]; u16 patterns[n_patterns][h][w]
//       OUT: f64 offsets and coefs of every pattern, in pattern order, from the
//            call sequence of the reference's file_processor
//            (src/process_files.hpp:98-233): load workers on threads calling
//            transfer_pic_to_device_async from pinned rasters, one thread that
//            waits with cudaStreamSynchronize(offs.in_stream) and calls
//            get_offset_core, one thread that calls finalize
//   shim_driver hooks MODE OUT
//       the sequence of the reference's test/cross_corr_fft_test.cpp:8-46 on a
//       gpu_offset<double, uint16_t> of mode MODE: get_cu_pic(), get_cu_temp(),
//       cross_corr_fft(); OUT: the 8 x 8 f64 correlation map
#include <cuda_runtime.h>

#include <atomic>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <iostream>
#include <mutex>
#include <thread>
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

// A bounded FIFO used as the reference's concurrent_queue is
// (src/concurrent_queue.hpp): push blocks while `capacity` items are queued,
// the consumer reads front() and pops only when it is done with the item.
template <typename V> class fifo {
    std::deque<V> q_;
    std::mutex m_;
    std::condition_variable cv_;
    const size_t cap_;

public:
    explicit fifo(size_t capacity) : cap_(capacity) {}
    void push(V v)
    {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return q_.size() < cap_; });
        q_.push_back(v);
        cv_.notify_all();
    }
    V front()
    {
        std::unique_lock<std::mutex> lk(m_);
        cv_.wait(lk, [&] { return !q_.empty(); });
        return q_.front();
    }
    void pop()
    {
        std::lock_guard<std::mutex> lk(m_);
        q_.pop_front();
        cv_.notify_all();
    }
};

void cuda_check(cudaError_t e)
{
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}

template <typename T>
int files(uint32_t w, uint32_t h, const std::vector<emida::size2_t> &begins, uint32_t batch,
          emida::cross_policy policy, int s, int mode, uint32_t n_patterns, uint32_t load_workers,
          const std::vector<uint16_t> &ref_in, const std::vector<uint16_t> &pics, FILE *out)
{
    using namespace emida;
    struct offs_job {
        esize_t batch_files, c, buffer_index;
    };
    struct fin_job {
        data_index<T> *maxes_i;
        T *neighbors;
        esize_t batch_files, c;
    };
    const size_t area = (size_t)w * h, n_rois = begins.size();
    gpu_offset<T, uint16_t> offs({w, h}, &begins, {64, 64}, {127, 127}, batch, policy, s,
                                 load_workers * 2, mode);
    std::vector<uint16_t> initial(ref_in);
    offs.allocate_memory(initial.data());
    const size_t total_slices = n_rois * batch;
    fin_job jobs[2];
    for (auto &j : jobs) {
        cuda_check(cudaMallocHost((void **)&j.maxes_i, total_slices * sizeof(data_index<T>)));
        cuda_check(cudaMallocHost((void **)&j.neighbors, total_slices * s * s * sizeof(T)));
    }
    std::vector<double> res_o(2 * n_rois * n_patterns), res_c(6 * n_rois * n_patterns);
    std::atomic<esize_t> current_file{0};
    fifo<offs_job> load_queue(load_workers);  // src/process_files.hpp:91
    fifo<fin_job *> fin_queue(1);
    std::vector<std::vector<uint16_t *>> rasters(load_workers);
    for (auto &rs : rasters) {
        rs.resize(load_workers + 1);
        for (auto &r : rs) cuda_check(cudaMallocHost((void **)&r, area * batch * sizeof(uint16_t)));
    }
    auto load_rasters = [&](uint32_t worker) {
        size_t ri = 0;
        esize_t c;
        while ((c = current_file.fetch_add(batch)) < n_patterns) {
            const esize_t batch_files = c + batch > n_patterns ? n_patterns - c : batch;
            uint16_t *next = rasters[worker][ri];
            std::memcpy(next, pics.data() + (size_t)c * area, batch_files * area * sizeof(uint16_t));
            const esize_t bi = offs.transfer_pic_to_device_async(next);
            load_queue.push({batch_files, c, bi});
            if (++ri >= rasters[worker].size()) ri = 0;
        }
    };
    const uint32_t n_batches = (n_patterns + batch - 1) / batch;
    std::thread comp([&] {
        fin_job *fjob = &jobs[0], *fjob_next = &jobs[1];
        for (uint32_t k = 0; k < n_batches; ++k) {
            const offs_job job = load_queue.front();
            cuda_check(cudaStreamSynchronize(offs.in_stream));  // src/process_files.hpp:196
            offs.get_offset_core(fjob->maxes_i, fjob->neighbors, job.buffer_index);
            load_queue.pop();
            fjob->c = job.c;
            fjob->batch_files = job.batch_files;
            fin_queue.push(fjob);
            std::swap(fjob, fjob_next);
        }
    });
    std::thread fin([&] {
        for (uint32_t k = 0; k < n_batches; ++k) {
            fin_job *j = fin_queue.front();
            auto r = offs.finalize(j->maxes_i, j->neighbors);
            for (size_t i = 0; i < (size_t)j->batch_files * n_rois; ++i) {
                const size_t g = (size_t)j->c * n_rois + i;
                res_o[2 * g] = r.offsets[i].x;
                res_o[2 * g + 1] = r.offsets[i].y;
                for (int q = 0; q < 6; ++q) res_c[6 * g + q] = r.coefs[i][q];
            }
            fin_queue.pop();
        }
    });
    std::vector<std::thread> loaders;
    for (uint32_t i = 1; i < load_workers; ++i) loaders.emplace_back(load_rasters, i);
    load_rasters(0);
    for (auto &t : loaders) t.join();
    comp.join();
    fin.join();
    fwrite(res_o.data(), sizeof(double), res_o.size(), out);
    fwrite(res_c.data(), sizeof(double), res_c.size(), out);
    for (auto &rs : rasters)
        for (auto *r : rs) cudaFreeHost(r);
    for (auto &j : jobs) {
        cudaFreeHost(j.maxes_i);
        cudaFreeHost(j.neighbors);
    }
    return 0;
}

int hooks(int mode, FILE *out)
{
    using namespace emida;
    // test/cross_corr_fft_test.cpp:10-38: an 8 x 8 zero-padded 4 x 4 ROI and an
    // 8 x 5 complex (8 x 10 real) buffer written straight into the spectra
    std::vector<double> in(64, 0.0), in_temp(80, 0.0);
    const double a[4][4] = {{1, 2, 3, 1}, {4, 5, 6, 1}, {7, 8, 9, 1}, {7, 8, 9, 1}};
    const double b[4][4] = {{6, 3, 2, 1}, {12, 23, 3, 1}, {1, 8, 9, 1}, {7, 8, 9, 1}};
    for (int y = 0; y < 4; ++y)
        for (int x = 0; x < 4; ++x) {
            in[y * 8 + x] = a[y][x];
            in_temp[y * 10 + x] = b[y][x];
        }
    size2_t slice_size{4, 4};
    std::vector<size2_t> begins{{0, 0}};
    gpu_offset<double, uint16_t> offs({10, 10}, &begins, slice_size, slice_size * 2 - 1, 1,
                                      CROSS_POLICY_FFT, 3, 1, mode);
    offs.allocate_memory(nullptr);
    cuda_check(cudaMemcpy(offs.get_cu_pic(), in.data(), in.size() * sizeof(double), cudaMemcpyHostToDevice));
    cuda_check(cudaMemcpy(offs.get_cu_temp(), in_temp.data(), in_temp.size() * sizeof(double),
                          cudaMemcpyHostToDevice));
    offs.cross_corr_fft();
    void *maps = nullptr;
    check_status(emida_gb_stage_buffers(offs.handle(), nullptr, nullptr, &maps));
    std::vector<double> res(64);
    cuda_check(cudaMemcpy(res.data(), maps, res.size() * sizeof(double), cudaMemcpyDeviceToHost));
    fwrite(res.data(), sizeof(double), res.size(), out);
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
        if (argc == 4 && !strcmp(argv[1], "files")) {
            FILE *in = fopen(argv[2], "rb"), *out = fopen(argv[3], "wb");
            if (!in || !out) return 2;
            std::vector<uint32_t> hdr, raw;
            if (!read_vec(in, hdr, 10)) return 2;
            const uint32_t w = hdr[0], h = hdr[1], n_rois = hdr[2], batch = hdr[3];
            const uint32_t n_patterns = hdr[8], load_workers = hdr[9];
            if (!read_vec(in, raw, 2 * (size_t)n_rois)) return 2;
            std::vector<emida::size2_t> begins(n_rois);
            for (uint32_t r = 0; r < n_rois; ++r) begins[r] = {raw[2 * r], raw[2 * r + 1]};
            std::vector<uint16_t> ref, pics;
            if (!read_vec(in, ref, (size_t)w * h) || !read_vec(in, pics, (size_t)n_patterns * w * h))
                return 2;
            const auto policy = hdr[4] ? emida::CROSS_POLICY_FFT : emida::CROSS_POLICY_BRUTE;
            const int rc = hdr[5] ? files<float>(w, h, begins, batch, policy, (int)hdr[6], (int)hdr[7],
                                                 n_patterns, load_workers, ref, pics, out)
                                  : files<double>(w, h, begins, batch, policy, (int)hdr[6], (int)hdr[7],
                                                  n_patterns, load_workers, ref, pics, out);
            fclose(in);
            fclose(out);
            return rc;
        }
        if (argc == 4 && !strcmp(argv[1], "hooks")) {
            FILE *out = fopen(argv[3], "wb");
            if (!out) return 2;
            const int rc = hooks(atoi(argv[2]), out);
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
    std::cerr << "usage: shim_driver validate | run IN OUT | pair IN OUT | files IN OUT | hooks MODE OUT\n";
    return 2;
}
