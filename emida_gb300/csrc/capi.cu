// capi.cu -- the C ABI (include/emida_gb.h): a handle that owns the device
// buffers, streams and resident reference spectra of one ROI layout, the
// host-side pieces of the reference's gpu_offset (src/gpu_offset.hpp:48-326),
// and the per-stage launch exports.
#include <cuda.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "deformation.cuh"
#include "fft.cuh"
#include "handle.cuh"
#include "ptx.cuh"

using namespace emida_gb;
using namespace emida_gb::host;

namespace {
thread_local std::string g_last_error;
}  // namespace

namespace emida_gb {
namespace host {

int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

}  // namespace host
}  // namespace emida_gb

namespace {

// ---- exact least-squares matrix ---------------------------------------------
// (A^T A)^-1 A^T for A rows (1, x, y, x^2, xy, y^2), x fastest
// (src/subpixel_max.hpp:42-67): Gauss-Jordan over exact rationals, one
// rounding per entry, which gives the same doubles as the reference's
// tables of src/subpixel_max.cpp:22-58.
struct q128 {
    __int128 n, d;
};
__int128 gcd_i(__int128 a, __int128 b)
{
    if (a < 0) a = -a;
    if (b < 0) b = -b;
    while (b != 0) {
        __int128 r = a % b;
        a = b;
        b = r;
    }
    return a;
}
q128 q_make(__int128 n, __int128 d)
{
    if (d < 0) {
        n = -n;
        d = -d;
    }
    __int128 g = gcd_i(n, d);
    if (g > 1) {
        n /= g;
        d /= g;
    }
    return q128{n, d};
}
q128 q_mul(q128 a, q128 b)
{
    q128 x = q_make(a.n, b.d), y = q_make(b.n, a.d);
    return q_make(x.n * y.n, x.d * y.d);
}
q128 q_sub(q128 a, q128 b) { return q_make(a.n * b.d - b.n * a.d, a.d * b.d); }
q128 q_div(q128 a, q128 b) { return q_mul(a, q_make(b.d, b.n)); }

}  // namespace

int emida_gb::host::lstsq_matrix(int s, double *out)
{
    if (s != 3 && s != 5 && s != 7 && s != 9) return -1;
    const int np = s * s, cols = 6 + np;
    std::vector<q128> M(6 * cols);
    auto at = [&](int r, int c) -> q128 & { return M[r * cols + c]; };
    auto feat = [&](int k, int f) -> long long {
        const long long x = k % s, y = k / s;
        const long long v[6] = {1, x, y, x * x, x * y, y * y};
        return v[f];
    };
    for (int i = 0; i < 6; ++i) {
        for (int j = 0; j < 6; ++j) {
            long long acc = 0;
            for (int k = 0; k < np; ++k) acc += feat(k, i) * feat(k, j);
            at(i, j) = q_make(acc, 1);
        }
        for (int k = 0; k < np; ++k) at(i, 6 + k) = q_make(feat(k, i), 1);
    }
    for (int c = 0; c < 6; ++c) {
        int piv = c;
        while (piv < 6 && at(piv, c).n == 0) ++piv;
        if (piv == 6) return -1;
        if (piv != c)
            for (int j = 0; j < cols; ++j) std::swap(at(c, j), at(piv, j));
        const q128 p = at(c, c);
        for (int j = 0; j < cols; ++j) at(c, j) = q_div(at(c, j), p);
        for (int i = 0; i < 6; ++i) {
            if (i == c || at(i, c).n == 0) continue;
            const q128 f = at(i, c);
            for (int j = 0; j < cols; ++j) at(i, j) = q_sub(at(i, j), q_mul(f, at(c, j)));
        }
    }
    for (int i = 0; i < 6; ++i)
        for (int k = 0; k < np; ++k) out[i * np + k] = (double)at(i, 6 + k).n / (double)at(i, 6 + k).d;
    return 0;
}

namespace {

// Host fit in the reference's operation order (src/subpixel_max.hpp:14-29, :76-97).
// This file is built with -ffp-contract=off, so each product and sum rounds once.
void host_fit(const double *mat, const double *v, int s, double *coef, double &x, double &y)
{
    const int np = s * s;
    for (int j = 0; j < 6; ++j) {
        double acc = 0;
        for (int k = 0; k < np; ++k) acc += mat[j * np + k] * v[k];
        coef[j] = acc;
    }
    const double b = coef[1], c = coef[2], d = coef[3], e = coef[4], f = coef[5];
    y = (b * e - 2 * c * d) / (4 * f * d - e * e);
    x = (-e * y - b) / (2 * d);
}

}  // namespace

// cuTensorMapEncodeTiled through the runtime's driver entry point (no libcuda link).
encode_fn emida_gb::host::get_encoder()
{
    static encode_fn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<encode_fn>(p);
    });
    return fn;
}



namespace {

template <typename T> std::vector<T> hann_host(uint32_t n)
{
    // src/host_helpers.hpp:29-37: FP64 formula, cast to T
    const double PI = 3.14159265358979323846;
    std::vector<T> v(n);
    for (uint32_t i = 0; i < n; ++i) v[i] = (T)(0.5 * (1 - std::cos(2 * PI * i / (double)(n - 1))));
    return v;
}

}  // namespace

int emida_gb::host::upload_hann(emida_gb_handle *h, void **dst, uint32_t nx, uint32_t ny)
{
    if (h->dbl) {
        auto x = hann_host<double>(nx), y = hann_host<double>(ny);
        x.insert(x.end(), y.begin(), y.end());
        CKS(h->alloc(dst, x.size() * sizeof(double)));
        CK(cudaMemcpy(*dst, x.data(), x.size() * sizeof(double), cudaMemcpyHostToDevice));
    } else {
        auto x = hann_host<float>(nx), y = hann_host<float>(ny);
        x.insert(x.end(), y.begin(), y.end());
        CKS(h->alloc(dst, x.size() * sizeof(float)));
        CK(cudaMemcpy(*dst, x.data(), x.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    return EMIDA_GB_OK;
}

int emida_gb::host::upload_twiddles(emida_gb_handle *h, void **dst, uint32_t n)
{
    const double PI = 3.14159265358979323846;
    if (h->dbl) {
        std::vector<double2> w(n);
        for (uint32_t j = 0; j < n; ++j)
            w[j] = make_double2(std::cos(2 * PI * j / n), -std::sin(2 * PI * j / n));
        CKS(h->alloc(dst, n * sizeof(double2)));
        CK(cudaMemcpy(*dst, w.data(), n * sizeof(double2), cudaMemcpyHostToDevice));
    } else {
        std::vector<float2> w(n);
        for (uint32_t j = 0; j < n; ++j)
            w[j] = make_float2((float)std::cos(2 * PI * j / n), (float)-std::sin(2 * PI * j / n));
        CKS(h->alloc(dst, n * sizeof(float2)));
        CK(cudaMemcpy(*dst, w.data(), n * sizeof(float2), cudaMemcpyHostToDevice));
    }
    return EMIDA_GB_OK;
}

fft_tables emida_gb::host::tables(const emida_gb_handle *h)
{
    return fft_tables{h->d_tw_row, h->d_tw_col, h->w2, h->h2};
}

// The staged pipeline for `pats` patterns from `pics` (<= B patterns):
// src/gpu_offset.hpp:234-278 stage by stage.
int emida_gb::host::run_plain_chunk(emida_gb_handle *h, const void *pics, uint32_t pats, void *maxes, void *neigh,
                    double *offsets, double *coefs, cudaStream_t st, const void *const *ptrs,
                    const uint32_t *out_base, void *maxes_out)
{
    const uint32_t n = pats * h->S;
    const int pol = h->fft ? POLICY_FFT : POLICY_BRUTE;
    CK(run_sums(pics, h->in_f64 ? IN_F64 : IN_U16, h->src, h->d_begins, h->S, h->slice, pats,
                h->d_sums, st, ptrs));
    CK(run_prepare(pics, h->in_f64 ? IN_F64 : IN_U16, h->dbl, h->d_prep, h->d_hann, h->d_sums,
                   h->d_begins, h->src, h->slice, h->prep_size(), h->S, pats, st, ptrs));
    if (h->fft) {
        CK(run_fft_r2c(h->d_prep, h->d_spec, n, tables(h), h->dbl, st));
        CK(run_hadamard(h->d_spec, h->d_ref_spec, h->h2 * h->half, h->S, pats, h->dbl, st));
        CK(run_fft_c2r(h->d_spec, h->d_map, n, tables(h), h->dbl, st));
    } else {
        CK(run_cross_corr(h->d_prep, h->d_ref_prep, h->d_map, h->dbl, h->slice, h->cross, h->S,
                          pats, st));
    }
    void *mx = maxes ? maxes : h->d_maxes;
    void *nb = neigh ? neigh : h->d_neigh;
    CK(run_maxarg(h->d_map, h->map_size(), n, mx, h->dbl, st));
    CK(run_extract_neighbors(h->d_map, mx, nb, h->p.fitsize, h->cross, n, pol, h->dbl, st));
    if (offsets)
        CK(run_fit(nb, mx, n, h->p.fitsize, h->cross, pol, h->d_lstsq, h->dbl, offsets, coefs, st,
                   out_base, h->S, maxes_out));
    return EMIDA_GB_OK;
}

int emida_gb::host::run_fused(emida_gb_handle *h, const void *pics, uint32_t pats, void *maxes, void *neigh,
              double *offsets, double *coefs, cudaStream_t st, const batch_view *view, int grid, uint32_t *err)
{
    const size2 src = view ? view->src : h->src;
    fused_args a{};
    a.pics = pics;
    a.src_w = src.x;
    a.src_h = src.y;
    a.begins = view ? view->begins : h->d_begins;
    a.n_rois = h->S;
    a.n_pairs = pats * h->S;
    a.side = h->slice.x;
    a.ref_spec = h->d_ref_spec_cm;
    a.hann = h->d_hann_fused;
    a.twiddles = h->d_tw_row;
    a.lstsq = h->d_lstsq;
    a.fitsize = h->p.fitsize;
    // the fused kernel always writes offsets; offsets_core passes none
    a.offsets = offsets ? offsets : h->d_offsets;
    a.coefs = coefs;
    a.maxes = maxes;
    a.neigh = neigh;
    a.err = err ? err : h->d_err;
    // the handle's own compute streams order their launches: a queue each
    a.pair_queue = st == h->comp ? h->d_queues : (h->comp_alt && st == h->comp_alt) ? h->d_queues + 2 : nullptr;
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    a.stage = STAGE_PLAIN;
    bool on_device = true;
    CKS(pattern_location(pics, on_device));
    if (on_device && !h->in_f64 && (src.x % 8) == 0 && ((uintptr_t)pics % 16) == 0) {
        if (encode_fn enc = get_encoder()) {
            const cuuint64_t dims[3] = {src.x, src.y, pats};
            const cuuint64_t strides[2] = {(cuuint64_t)src.x * 2, (cuuint64_t)src.x * src.y * 2};
            const cuuint32_t box[3] = {(h->slice.x + 14) & ~7u, fused_box_rows(h->w2, h->slice.y), 1};
            const cuuint32_t estr[3] = {1, 1, 1};
            if (enc(&map, CU_TENSOR_MAP_DATA_TYPE_UINT16, 3, const_cast<void *>(pics), dims,
                    strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
                a.stage = STAGE_TMA;
        }
    }
    // pinned host patterns: cp.async chunks over the host link
    if (a.stage == STAGE_PLAIN && !h->in_f64 && (src.x % 8) == 0 && ((uintptr_t)pics % 16) == 0)
        a.stage = STAGE_ASYNC;
    CK(launch_fused(h->w2, h->dbl, h->in_f64, a, &map, grid, st));
    return EMIDA_GB_OK;
}

int emida_gb::host::run_tensor(emida_gb_handle *h, const void *pics, uint32_t pats, void *maxes, void *neigh,
               double *offsets, double *coefs, cudaStream_t st, const batch_view *view, int grid, uint32_t *err)
{
    brute_tc_args a{};
    a.pics = static_cast<const uint16_t *>(pics);
    a.src_w = view ? view->src.x : h->src.x;
    a.src_h = view ? view->src.y : h->src.y;
    a.begins = view ? view->begins : h->d_begins;
    a.n_rois = h->S;
    a.n_patterns = pats;
    a.ref_prep = h->d_ref_prep64;
    a.hann = h->d_hann64;
    a.lstsq = h->d_lstsq;
    a.fitsize = h->p.fitsize;
    a.offsets = offsets ? offsets : h->d_offsets;
    a.coefs = coefs;
    a.maxes = maxes;
    a.neigh = static_cast<float *>(neigh);
    a.err = err ? err : h->d_err;
    CK(launch_brute_tc(a, grid, st));
    return EMIDA_GB_OK;
}

int emida_gb::host::run_any(emida_gb_handle *h, const void *pics, uint32_t pats, void *maxes, void *neigh,
            double *offsets, double *coefs, cudaStream_t st, const batch_view *view, int grid, uint32_t *err)
{
    if (h->mode == EMIDA_GB_MODE_FUSED)
        return run_fused(h, pics, pats, maxes, neigh, offsets, coefs, st, view, grid, err);
    if (h->mode == EMIDA_GB_MODE_TENSOR)
        return run_tensor(h, pics, pats, maxes, neigh, offsets, coefs, st, view, grid, err);
    if (view) return fail(EMIDA_GB_UNSUPPORTED, "the staged form reads whole patterns only");
    const size_t pat_bytes = (size_t)h->src.x * h->src.y * h->in_elem;
    const size_t s2 = (size_t)h->p.fitsize * h->p.fitsize;
    for (uint32_t done = 0; done < pats; done += h->B) {
        const uint32_t c = pats - done < h->B ? pats - done : h->B;
        const size_t r0 = (size_t)done * h->S;
        CKS(run_plain_chunk(h, (const char *)pics + done * pat_bytes, c,
                            maxes ? (char *)maxes + r0 * h->di_elem : nullptr,
                            neigh ? (char *)neigh + r0 * s2 * h->t_elem : nullptr,
                            offsets ? offsets + 2 * r0 : nullptr, coefs ? coefs + 6 * r0 : nullptr,
                            st));
    }
    return EMIDA_GB_OK;
}

int emida_gb::host::pattern_location(const void *patterns, bool &on_device)
{
    cudaPointerAttributes pa{};
    CK(cudaPointerGetAttributes(&pa, patterns));
    if (pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged) {
        on_device = true;
        return EMIDA_GB_OK;
    }
    if (pa.type == cudaMemoryTypeHost) {
        on_device = false;
        return EMIDA_GB_OK;
    }
    return fail(EMIDA_GB_INVALID_ARGUMENT, "patterns must be in device memory or pinned host memory");
}

int emida_gb::host::copy_patterns(emida_gb_handle *h, void *dst, const void *src, uint32_t patterns,
                                  cudaStream_t st)
{
    const size_t row = (size_t)h->src.x * h->in_elem, pat = row * h->src.y;
    if (h->bands.size() == 1 && h->bands[0].first == 0 && h->bands[0].second == h->src.y) {
        CK(cudaMemcpyAsync(dst, src, pat * patterns, cudaMemcpyHostToDevice, st));
        return EMIDA_GB_OK;
    }
    for (const auto &b : h->bands)
        CK(cudaMemcpy2DAsync((char *)dst + b.first * row, pat, (const char *)src + b.first * row, pat,
                             b.second * row, patterns, cudaMemcpyHostToDevice, st));
    return EMIDA_GB_OK;
}

namespace {

// Merged row bands of the ROIs; one full band when they cover 90 % of the rows.
void row_bands(emida_gb_handle *h)
{
    std::vector<std::pair<uint32_t, uint32_t>> iv;  // [start, end)
    for (uint32_t r = 0; r < h->S; ++r) iv.push_back({h->begins[2 * r + 1], h->begins[2 * r + 1] + h->slice.y});
    std::sort(iv.begin(), iv.end());
    std::vector<std::pair<uint32_t, uint32_t>> merged;
    for (const auto &v : iv) {
        if (!merged.empty() && v.first <= merged.back().second)
            merged.back().second = std::max(merged.back().second, v.second);
        else
            merged.push_back(v);
    }
    uint64_t covered = 0;
    for (const auto &m : merged) covered += m.second - m.first;
    h->bands.clear();
    if (covered * 10 >= (uint64_t)h->src.y * 9) {
        h->bands.push_back({0, h->src.y});
        return;
    }
    for (const auto &m : merged) h->bands.push_back({m.first, m.second - m.first});
}

}  // namespace

int emida_gb::host::device_flags_status(uint32_t err)
{
    if (!err) return EMIDA_GB_OK;
    return fail(EMIDA_GB_DEVICE_CHECK, "device check failed (flags 0x%x%s%s)", err,
                (err & DEV_ERR_TMA_TIMEOUT) ? ": TMA wait ran out" : "",
                (err & DEV_ERR_WAIT_TIMEOUT) ? ": pipeline wait ran out" : "");
}

int emida_gb::host::check_device_error(emida_gb_handle *h, uint32_t *word)
{
    uint32_t *w = word ? word : h->d_err;
    uint32_t err = 0;
    CK(cudaMemcpy(&err, w, sizeof err, cudaMemcpyDeviceToHost));
    if (err) {
        // the handle's streams do not wait for the legacy stream: the clear
        // completes here, before any later launch can set the word again
        CK(cudaMemsetAsync(w, 0, sizeof err, cudaStreamLegacy));
        CK(cudaStreamSynchronize(cudaStreamLegacy));
    }
    return device_flags_status(err);
}

namespace {

int validate(const emida_gb_params *p)
{
    if (!p) return fail(EMIDA_GB_INVALID_ARGUMENT, "null parameters");
    if (p->src_w == 0 || p->src_h == 0) return fail(EMIDA_GB_INVALID_ARGUMENT, "empty pattern size");
    if (p->n_rois == 0 || !p->begins) return fail(EMIDA_GB_INVALID_ARGUMENT, "no ROIs");
    if (p->slice_w < 2 || p->slice_h < 2) return fail(EMIDA_GB_INVALID_ARGUMENT, "ROI smaller than 2x2");
    if (p->batch_size == 0) return fail(EMIDA_GB_INVALID_ARGUMENT, "batchsize must be greater than 0");
    // pair counts and pair indices are 32-bit on the device
    if ((uint64_t)p->n_rois * p->batch_size > 0x7fffffffu)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "ROIs x batchsize (%llu) exceeds 2^31 - 1",
                    (unsigned long long)p->n_rois * p->batch_size);
    if (p->policy != EMIDA_GB_BRUTE && p->policy != EMIDA_GB_FFT)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "invalid cross policy %d", p->policy);
    if (p->precision != EMIDA_GB_DOUBLE && p->precision != EMIDA_GB_FLOAT)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "invalid precision %d", p->precision);
    if (p->fitsize != 3 && p->fitsize != 5 && p->fitsize != 7 && p->fitsize != 9)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "Wrong fitting size.");
    if (p->in_type != EMIDA_GB_IN_U16 && p->in_type != EMIDA_GB_IN_F64)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "invalid input type %d", p->in_type);
    for (uint32_t r = 0; r < p->n_rois; ++r)
        if ((uint64_t)p->begins[2 * r] + p->slice_w > p->src_w ||
            (uint64_t)p->begins[2 * r + 1] + p->slice_h > p->src_h)
            return fail(EMIDA_GB_INVALID_ARGUMENT, "A slice out of bounds (ROI %u)", r);
    if (p->policy == EMIDA_GB_BRUTE) {
        if (p->cross_w == 0 || p->cross_h == 0 || p->cross_w > 2 * p->slice_w - 1 ||
            p->cross_h > 2 * p->slice_h - 1)
            return fail(EMIDA_GB_INVALID_ARGUMENT,
                        "cross size must be lesser or equal to slice_size * 2 - 1");
    } else if (p->slice_w != p->slice_h) {
        return fail(EMIDA_GB_UNSUPPORTED, "the FFT policy needs square ROIs");
    }
    if (p->mode < EMIDA_GB_MODE_AUTO || p->mode > EMIDA_GB_MODE_TENSOR)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "invalid mode %d", p->mode);
    if (p->mode == EMIDA_GB_MODE_TENSOR &&
        (p->policy != EMIDA_GB_BRUTE || p->precision != EMIDA_GB_FLOAT || p->in_type != EMIDA_GB_IN_U16 ||
         p->slice_w != BRUTE_TC_SIDE || p->slice_h != BRUTE_TC_SIDE || p->cross_w != BRUTE_TC_CROSS ||
         p->cross_h != BRUTE_TC_CROSS))
        return fail(EMIDA_GB_UNSUPPORTED,
                    "the tensor-core form takes the brute policy, float precision, uint16 input, "
                    "64x64 ROIs and a 127x127 lag window");
    return EMIDA_GB_OK;
}

}  // namespace

namespace {

// One warp waits on phase 0 of an mbarrier that expects one arrival and gets
// none: the bounded wait gives up after `budget` cycles and records it.
__global__ void k_selftest_wait(uint32_t *err, long long budget)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) emida_gb::ptx::mbar_init(&bar, 1);
    __syncthreads();
    const bool done = emida_gb::ptx::mbar_wait_for(&bar, 0, budget);
    if (!done && threadIdx.x == 0) atomicOr(err, DEV_ERR_WAIT_TIMEOUT);
    __syncthreads();
}

}  // namespace

namespace {

// The staged form's buffers behind the test hooks (src/gpu_offset.hpp:303-325):
// the staged handle's own, or for the fused and tensor forms, which keep no
// such buffers, a set at the staged sizes made on first use.  With the FFT
// policy and a reference registered, the set's reference spectra are computed
// from the registered pattern.
int stage_hooks(emida_gb_handle *h)
{
    auto &k = h->hk;
    if (k.ready) return EMIDA_GB_OK;
    if (h->mode == EMIDA_GB_MODE_PLAIN) {
        k.pic = h->d_prep;
        k.temp = h->fft ? h->d_ref_spec : h->d_ref_prep;
        k.spec = h->d_spec;
        k.map = h->d_map;
        k.tw_row = h->d_tw_row;
        k.tw_col = h->d_tw_col;
        k.ready = true;
        return EMIDA_GB_OK;
    }
    if (!h->fft) {
        // the tensor form: FP32 prepared patterns and brute maps; its FP32
        // reference ROIs are the ones set_reference prepares
        CKS(h->alloc(&k.pic, (size_t)h->slice.x * h->slice.y * h->N * h->t_elem, true));
        CKS(h->alloc(&k.map, (size_t)h->cross.x * h->cross.y * h->N * h->t_elem, true));
        k.temp = h->d_ref_prep;
        k.ready = true;
        return EMIDA_GB_OK;
    }
    const uint32_t w2 = 2 * h->slice.x, h2 = 2 * h->slice.y, half = w2 / 2 + 1;
    CKS(h->alloc(&k.pic, (size_t)w2 * h2 * h->N * h->t_elem, true));
    CKS(h->alloc(&k.ref_prep, (size_t)w2 * h2 * h->S * h->t_elem, true));
    CKS(h->alloc(&k.temp, (size_t)h2 * half * h->S * h->c_elem, true));
    CKS(h->alloc(&k.spec, (size_t)h2 * half * h->N * h->c_elem));
    CKS(h->alloc(&k.map, (size_t)w2 * h2 * h->N * h->t_elem, true));
    CKS(upload_twiddles(h, &k.tw_row, w2));
    CKS(upload_twiddles(h, &k.tw_col, h2));
    k.ready = true;
    if (h->ref_set) CKS(stage_hooks_reference(h));
    return EMIDA_GB_OK;
}

}  // namespace

int emida_gb::host::stage_hooks_reference(emida_gb_handle *h)
{
    auto &k = h->hk;
    if (!k.ready || !k.ref_prep) return EMIDA_GB_OK;
    const uint32_t w2 = 2 * h->slice.x, h2 = 2 * h->slice.y;
    const int in_type = h->in_f64 ? IN_F64 : IN_U16;
    CK(run_prepare(h->d_ref_in, in_type, h->dbl, k.ref_prep, h->d_hann, h->d_sums_ref, h->d_begins,
                   h->src, h->slice, size2{w2, h2}, h->S, 1, h->comp));
    CK(run_fft_r2c(k.ref_prep, k.temp, h->S, fft_tables{k.tw_row, k.tw_col, w2, h2}, h->dbl, h->comp));
    CK(cudaStreamSynchronize(h->comp));
    return EMIDA_GB_OK;
}

extern "C" {

const char *emida_gb_last_error(void) { return g_last_error.c_str(); }
const char *emida_gb_version(void) { return "emida-gb300 0.1 (sm_103a)"; }

int emida_gb_lstsq_matrix(int s, double *out)
{
    if (!out || lstsq_matrix(s, out) != 0) return fail(EMIDA_GB_INVALID_ARGUMENT, "Wrong fitting size.");
    return EMIDA_GB_OK;
}

int emida_gb_subpixel_max(const double *neigh, int s, uint32_t n, double *sub, double *coefs)
{
    double mat[6 * 81];
    if (lstsq_matrix(s, mat) != 0) return fail(EMIDA_GB_INVALID_ARGUMENT, "Wrong fitting size.");
    for (uint32_t i = 0; i < n; ++i) {
        double c[6], x, y;
        host_fit(mat, neigh + (size_t)i * s * s, s, c, x, y);
        sub[2 * i] = x;
        sub[2 * i + 1] = y;
        if (coefs) std::memcpy(coefs + 6 * (size_t)i, c, sizeof c);
    }
    return EMIDA_GB_OK;
}

int emida_gb_create(const emida_gb_params *p, emida_gb_handle **out)
{
    return create_handle(p, 0, out);
}

}  // extern "C"

int emida_gb::host::create_handle(const emida_gb_params *p, uint32_t fused_len, emida_gb_handle **out)
{
    if (!out) return fail(EMIDA_GB_INVALID_ARGUMENT, "null output handle");
    *out = nullptr;
    CKS(validate(p));
    auto *h = new emida_gb_handle();
    h->p = *p;
    h->begins.assign(p->begins, p->begins + 2 * (size_t)p->n_rois);
    h->p.begins = h->begins.data();
    if (h->p.in_buffers == 0) h->p.in_buffers = 1;
    h->dbl = p->precision == EMIDA_GB_DOUBLE;
    h->in_f64 = p->in_type == EMIDA_GB_IN_F64;
    h->fft = p->policy == EMIDA_GB_FFT;
    h->src = size2{p->src_w, p->src_h};
    h->slice = size2{p->slice_w, p->slice_h};
    h->S = p->n_rois;
    h->B = p->batch_size;
    h->N = h->S * h->B;
    h->in_elem = h->in_f64 ? 8 : 2;
    h->t_elem = h->dbl ? 8 : 4;
    h->c_elem = 2 * h->t_elem;
    h->di_elem = h->dbl ? sizeof(data_index<double>) : sizeof(data_index<float>);
    if (h->fft) {
        h->w2 = 2 * p->slice_w;
        h->h2 = 2 * p->slice_h;
        h->half = h->w2 / 2 + 1;
        h->cross = size2{2 * p->slice_w - 1, 2 * p->slice_h - 1};
    } else {
        h->cross = size2{p->cross_w, p->cross_h};
    }
    // The fused kernel takes square ROIs up to 96 pixels (64 in FP64); a ROI
    // whose 2*side is not one of its transform lengths is zero-padded into the
    // next one, which leaves every lag of the 2*side-1 window unchanged.
    uint32_t fn = h->fft ? fused_size_for(p->slice_w, h->dbl, h->in_f64) : 0;
    if (fused_len && fn) {
        // a longer fused transform chosen by the caller (the multi-layout autotuner)
        if (fused_len < 2 * p->slice_w || !fused_supported(fused_len, h->dbl, h->in_f64)) {
            delete h;
            return fail(EMIDA_GB_UNSUPPORTED, "no fused %u-point transform for ROI side %u", fused_len,
                        p->slice_w);
        }
        fn = fused_len;
    }
    const bool fusable = fn != 0;
    if (p->mode == EMIDA_GB_MODE_FUSED && !fusable) {
        delete h;
        return fail(EMIDA_GB_UNSUPPORTED,
                    "no fused kernel for this shape (FFT policy; ROI side <= 64 in FP64, <= 96 in FP32, "
                    "<= 128 in FP32 with uint16 input)");
    }
    h->mode = (p->mode == EMIDA_GB_MODE_PLAIN || !fusable) ? EMIDA_GB_MODE_PLAIN : EMIDA_GB_MODE_FUSED;
    if (p->mode == EMIDA_GB_MODE_TENSOR) h->mode = EMIDA_GB_MODE_TENSOR;
    row_bands(h);
    h->in_place_allowed = h->mode != EMIDA_GB_MODE_PLAIN &&
                          2 * (uint64_t)p->n_rois * p->slice_w * p->slice_h <= (uint64_t)p->src_w * p->src_h;
    h->gather_allowed = h->mode != EMIDA_GB_MODE_PLAIN && !h->in_f64 && p->src_w % 8 == 0 &&
                        (uint64_t)p->n_rois * p->slice_h * gather_width(p->slice_w) <=
                            (uint64_t)p->src_w * p->src_h;
    // a pattern of at most 2^31 16-byte chunks (chunk indices within a run
    // stay 32-bit), whose rows are whole chunks
    h->sm_copy_allowed = ((uint64_t)p->src_w * h->in_elem) % 16 == 0 &&
                         (uint64_t)p->src_w * p->src_h * h->in_elem / 16 <= 0x7fffffffu;
    // the fused and tensor forms leave CTA slots for the SM copy beside them
    h->ingest = h->sm_copy_allowed && h->mode != EMIDA_GB_MODE_PLAIN ? EMIDA_GB_INGEST_SM_COPY
                                                                     : EMIDA_GB_INGEST_COPY;
    if (h->mode == EMIDA_GB_MODE_FUSED) {
        // the resident reference spectra are computed at the fused length
        h->w2 = h->h2 = fn;
        h->half = fn / 2 + 1;
    }

    auto bail = [&](int st) {
        emida_gb_destroy(h);
        return st;
    };
    int st;
#define TRY(expr)                                                                           \
    if ((st = (expr)) != EMIDA_GB_OK) return bail(st);
    TRY([&]() -> int { CK(cudaGetDevice(&h->device)); return EMIDA_GB_OK; }());
    TRY([&]() -> int {
        // the input stream's copy CTAs are dispatched ahead of a path's
        // pending CTAs when two batches' paths overlap
        int least = 0;
        int greatest = 0;
        CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CK(cudaStreamCreateWithPriority(&h->in_stream, cudaStreamNonBlocking, greatest));
        CK(cudaStreamCreateWithFlags(&h->out_stream, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&h->comp, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->comp_done, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&h->out_done, cudaEventDisableTiming));
        h->in_done.resize(h->p.in_buffers);
        for (auto &e : h->in_done) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        h->in_used.resize(h->p.in_buffers);
        for (auto &e : h->in_used) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        return EMIDA_GB_OK;
    }());
    const size_t pat_bytes = (size_t)h->src.x * h->src.y * h->in_elem;
    h->d_in.resize(h->p.in_buffers);
    for (auto &b : h->d_in) TRY(h->alloc(&b, pat_bytes * h->B));
    TRY(h->alloc(&h->d_ref_in, pat_bytes));
    TRY(h->alloc((void **)&h->d_begins, sizeof(uint2) * h->S));
    TRY([&]() -> int {
        CK(cudaMemcpy(h->d_begins, h->begins.data(), sizeof(uint2) * h->S, cudaMemcpyHostToDevice));
        return EMIDA_GB_OK;
    }());
    if (h->gather_allowed) {
        std::vector<uint32_t> compact(2 * (size_t)h->S);
        for (uint32_t r = 0; r < h->S; ++r) {
            compact[2 * r] = h->begins[2 * r] & 7u;
            compact[2 * r + 1] = r * h->slice.y;
        }
        TRY(h->alloc((void **)&h->d_begins_compact, sizeof(uint2) * h->S));
        TRY([&]() -> int {
            CK(cudaMemcpy(h->d_begins_compact, compact.data(), sizeof(uint2) * h->S,
                          cudaMemcpyHostToDevice));
            return EMIDA_GB_OK;
        }());
    }
    if (h->sm_copy_allowed) {
        const uint32_t row16 = (uint32_t)(h->src.x * h->in_elem / 16);
        std::vector<uint2> runs;
        for (const auto &b : h->bands) runs.push_back(make_uint2(b.first * row16, b.second * row16));
        h->n_band_runs = (uint32_t)runs.size();
        TRY(h->alloc((void **)&h->d_band_runs, sizeof(uint2) * runs.size()));
        TRY([&]() -> int {
            CK(cudaMemcpy(h->d_band_runs, runs.data(), sizeof(uint2) * runs.size(), cudaMemcpyHostToDevice));
            return EMIDA_GB_OK;
        }());
    }
    TRY(upload_hann(h, &h->d_hann, h->slice.x, h->slice.y));
    const size_t sum_elem = h->in_f64 ? 8 : 4;
    TRY(h->alloc(&h->d_sums_ref, sum_elem * h->S));
    TRY(h->alloc((void **)&h->d_err, sizeof(uint32_t), true));
    TRY(h->alloc((void **)&h->d_queues, 4 * sizeof(uint32_t), true));
    h->lstsq.resize(6 * (size_t)p->fitsize * p->fitsize);
    lstsq_matrix(p->fitsize, h->lstsq.data());
    TRY(h->alloc((void **)&h->d_lstsq, h->lstsq.size() * sizeof(double)));
    TRY([&]() -> int {
        CK(cudaMemcpy(h->d_lstsq, h->lstsq.data(), h->lstsq.size() * sizeof(double),
                      cudaMemcpyHostToDevice));
        return EMIDA_GB_OK;
    }());
    const size2 ps = h->prep_size();
    TRY(h->alloc(&h->d_ref_prep, (size_t)ps.x * ps.y * h->S * h->t_elem, true));
    if (h->fft) {
        TRY(upload_twiddles(h, &h->d_tw_row, h->w2));
        TRY(upload_twiddles(h, &h->d_tw_col, h->h2));
        TRY(h->alloc(&h->d_ref_spec, (size_t)h->h2 * h->half * h->S * h->c_elem));
    }
    const size_t s2 = (size_t)p->fitsize * p->fitsize;
    if (h->mode == EMIDA_GB_MODE_FUSED) {
        TRY(upload_hann(h, &h->d_hann_fused, h->slice.x, h->slice.y));
        TRY(h->alloc(&h->d_ref_spec_cm, (size_t)h->h2 * h->half * h->S * h->c_elem));
    } else if (h->mode == EMIDA_GB_MODE_TENSOR) {
        // FP64 windows and reference ROIs; no per-batch scratch
        h->dbl = true;
        TRY(upload_hann(h, (void **)&h->d_hann64, h->slice.x, h->slice.y));
        h->dbl = false;
        TRY(h->alloc((void **)&h->d_ref_prep64, (size_t)ps.x * ps.y * h->S * sizeof(double), true));
    } else {
        TRY(h->alloc(&h->d_sums, sum_elem * h->N));
        TRY(h->alloc(&h->d_prep, (size_t)ps.x * ps.y * h->N * h->t_elem, true));
        TRY(h->alloc(&h->d_map, (size_t)h->map_size() * h->N * h->t_elem));
        if (h->fft) TRY(h->alloc(&h->d_spec, (size_t)h->h2 * h->half * h->N * h->c_elem));
    }
    TRY(h->alloc(&h->d_maxes, h->di_elem * h->N));
    TRY(h->alloc(&h->d_neigh, s2 * h->N * h->t_elem));
    TRY(h->alloc((void **)&h->d_offsets, 2 * sizeof(double) * h->N));
    TRY(h->alloc((void **)&h->d_coefs, 6 * sizeof(double) * h->N));
#undef TRY
    *out = h;
    return EMIDA_GB_OK;
}

extern "C" {

int emida_gb_set_reference(emida_gb_handle *h, const void *ref)
{
    trace_range tr("emida_gb_set_reference");
    if (!h || !ref) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(h->mu);
    const size_t pat_bytes = (size_t)h->src.x * h->src.y * h->in_elem;
    CK(cudaMemcpyAsync(h->d_ref_in, ref, pat_bytes, cudaMemcpyHostToDevice, h->comp));
    const int in_type = h->in_f64 ? IN_F64 : IN_U16;
    CK(run_sums(h->d_ref_in, in_type, h->src, h->d_begins, h->S, h->slice, 1, h->d_sums_ref, h->comp));
    CK(run_prepare(h->d_ref_in, in_type, h->dbl, h->d_ref_prep, h->d_hann, h->d_sums_ref,
                   h->d_begins, h->src, h->slice, h->prep_size(), h->S, 1, h->comp));
    if (h->mode == EMIDA_GB_MODE_TENSOR)
        CK(run_prepare(h->d_ref_in, in_type, true, h->d_ref_prep64, h->d_hann64, h->d_sums_ref,
                       h->d_begins, h->src, h->slice, h->prep_size(), h->S, 1, h->comp));
    if (h->fft) {
        CK(run_fft_r2c(h->d_ref_prep, h->d_ref_spec, h->S, tables(h), h->dbl, h->comp));
        if (h->d_ref_spec_cm) {
            CK(run_spec_to_colmajor(h->d_ref_spec, h->d_ref_spec_cm, h->S, h->w2, h->h2, h->dbl,
                                    h->comp));
            // the fused kernels correlate the packed DC and Nyquist slot
            // directly, from the reference's row sums in column 0
            CK(run_ref_row_sums(h->d_ref_prep, h->d_ref_spec_cm, h->S, h->w2, h->dbl, h->comp));
        }
    }
    // the path's kernel is loaded now rather than at the first batch
    if (h->mode == EMIDA_GB_MODE_FUSED) CK(preload_fused(h->w2, h->dbl, h->in_f64));
    if (h->mode == EMIDA_GB_MODE_TENSOR) CK(preload_brute_tc());
    CK(cudaStreamSynchronize(h->comp));
    h->ref_set = true;
    return stage_hooks_reference(h);
}

int emida_gb_transfer_async(emida_gb_handle *h, const void *batch, uint32_t *buffer_index)
{
    trace_range tr("emida_gb_transfer_async");
    if (!h || !batch) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    const uint32_t i = h->in_next.fetch_add(1) % (uint32_t)h->d_in.size();
    // offsets_core returns before its kernels have read the buffer (the
    // reference's waits for the device): the copy waits for the last
    // offsets_core that read this buffer
    CK(cudaStreamWaitEvent(h->in_stream, h->in_used[i], 0));
    CKS(copy_patterns(h, h->d_in[i], batch, h->B, h->in_stream));
    CK(cudaEventRecord(h->in_done[i], h->in_stream));
    if (buffer_index) *buffer_index = i;
    return EMIDA_GB_OK;
}

int emida_gb_offsets_core(emida_gb_handle *h, uint32_t buffer_index, void *maxes_out,
                          void *neigh_out)
{
    trace_range tr("emida_gb_offsets_core");
    if (!h) return fail(EMIDA_GB_INVALID_ARGUMENT, "null handle");
    if (buffer_index >= h->d_in.size()) return fail(EMIDA_GB_INVALID_ARGUMENT, "bad buffer index");
    if (!h->ref_set) return fail(EMIDA_GB_INVALID_ARGUMENT, "reference pattern not set");
    std::lock_guard<std::mutex> lk(h->mu);
    CK(cudaStreamWaitEvent(h->comp, h->in_done[buffer_index], 0));
    // the previous call's copies of the maxima and neighbourhoods read the
    // buffers this call overwrites (the reference's kernels on the legacy
    // stream wait for its blocking output stream in the same way)
    CK(cudaStreamWaitEvent(h->comp, h->out_done, 0));
    CKS(run_any(h, h->d_in[buffer_index], h->B, h->d_maxes, h->d_neigh, nullptr, nullptr, h->comp));
    CK(cudaEventRecord(h->in_used[buffer_index], h->comp));
    CK(cudaEventRecord(h->comp_done, h->comp));
    CK(cudaStreamWaitEvent(h->out_stream, h->comp_done, 0));
    const size_t s2 = (size_t)h->p.fitsize * h->p.fitsize;
    if (maxes_out)
        CK(cudaMemcpyAsync(maxes_out, h->d_maxes, h->di_elem * h->N, cudaMemcpyDeviceToHost, h->out_stream));
    if (neigh_out)
        CK(cudaMemcpyAsync(neigh_out, h->d_neigh, s2 * h->t_elem * h->N, cudaMemcpyDeviceToHost,
                           h->out_stream));
    CK(cudaEventRecord(h->out_done, h->out_stream));
    return EMIDA_GB_OK;
}

int emida_gb_finalize(emida_gb_handle *h, const void *maxes, const void *neigh, double *offsets,
                      double *coefs)
{
    trace_range tr("emida_gb_finalize");
    if (!h || !maxes || !neigh || !offsets) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    CK(cudaStreamSynchronize(h->out_stream));
    CKS(check_device_error(h));
    const int s = h->p.fitsize, s2 = s * s, r = (s - 1) / 2;
    std::vector<double> v(s2);
    for (uint32_t i = 0; i < h->N; ++i) {
        uint32_t index;
        if (h->dbl) {
            index = reinterpret_cast<const data_index<double> *>(maxes)[i].index;
            for (int k = 0; k < s2; ++k) v[k] = reinterpret_cast<const double *>(neigh)[(size_t)i * s2 + k];
        } else {
            index = reinterpret_cast<const data_index<float> *>(maxes)[i].index;
            for (int k = 0; k < s2; ++k) v[k] = (double)reinterpret_cast<const float *>(neigh)[(size_t)i * s2 + k];
        }
        double c[6], sx, sy;
        host_fit(h->lstsq.data(), v.data(), s, c, sx, sy);
        uint32_t mx, my;
        if (h->fft) {
            const uint32_t iw = h->cross.x + 1, ih = h->cross.y + 1;
            mx = (index % iw + (iw - 1) / 2) % iw;
            my = (index / iw + (ih - 1) / 2) % ih;
        } else {
            mx = index % h->cross.x;
            my = index / h->cross.x;
        }
        offsets[2 * (size_t)i] = -((int)mx - ((int)h->cross.x / 2) - r + sx);
        offsets[2 * (size_t)i + 1] = -((int)my - ((int)h->cross.y / 2) - r + sy);
        if (coefs) std::memcpy(coefs + 6 * (size_t)i, c, sizeof c);
    }
    return EMIDA_GB_OK;
}

int emida_gb_get_offset(emida_gb_handle *h, const void *batch, double *offsets, double *coefs,
                        uint32_t *peaks)
{
    trace_range tr("emida_gb_get_offset");
    if (!h || !batch || !offsets) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    if (!h->ref_set) return fail(EMIDA_GB_INVALID_ARGUMENT, "reference pattern not set");
    std::lock_guard<std::mutex> lk(h->mu);
    CK(cudaStreamWaitEvent(h->comp, h->out_done, 0));  // offsets_core's copies read d_maxes, d_neigh
    CKS(copy_patterns(h, h->d_in[0], batch, h->B, h->comp));
    CKS(run_any(h, h->d_in[0], h->B, h->d_maxes, h->d_neigh, h->d_offsets, h->d_coefs, h->comp));
    CK(cudaMemcpyAsync(offsets, h->d_offsets, 2 * sizeof(double) * h->N, cudaMemcpyDeviceToHost, h->comp));
    if (coefs)
        CK(cudaMemcpyAsync(coefs, h->d_coefs, 6 * sizeof(double) * h->N, cudaMemcpyDeviceToHost, h->comp));
    std::vector<unsigned char> mx;
    if (peaks) {
        mx.resize(h->di_elem * h->N);
        CK(cudaMemcpyAsync(mx.data(), h->d_maxes, mx.size(), cudaMemcpyDeviceToHost, h->comp));
    }
    CK(cudaStreamSynchronize(h->comp));
    CKS(check_device_error(h));
    if (peaks)
        for (uint32_t i = 0; i < h->N; ++i)
            peaks[i] = h->dbl ? reinterpret_cast<const data_index<double> *>(mx.data())[i].index
                              : reinterpret_cast<const data_index<float> *>(mx.data())[i].index;
    return EMIDA_GB_OK;
}

// CTAs of the gather ingest: host reads over NVLink-C2C top out near 15 GB/s
// per SM, so 16 CTAs of 256 threads reach the link's rate for ROI rows
// (about 145 GB/s of ROI pixels against 211 GB/s for contiguous reads) when
// they run alone; beside the path's CTAs they run slower.
constexpr int GATHER_CTAS = 16;
constexpr int COPY_CTAS = 16;

static int ring_init(emida_gb_handle *h)
{
    if (!h->ring.empty()) return EMIDA_GB_OK;
    std::vector<emida_gb_handle::slot> ring(h->d_in.size());
    for (auto &r : ring) {
        CKS(h->alloc((void **)&r.d_offsets, 2 * sizeof(double) * h->N));
        CKS(h->alloc((void **)&r.d_coefs, 6 * sizeof(double) * h->N));
        CKS(h->alloc(&r.d_maxes, h->di_elem * h->N));
        CK(cudaMallocHost((void **)&r.h_offsets, 2 * sizeof(double) * h->N));
        CK(cudaMallocHost((void **)&r.h_coefs, 6 * sizeof(double) * h->N));
        CK(cudaMallocHost(&r.h_maxes, h->di_elem * h->N));
        CKS(h->alloc((void **)&r.d_err, sizeof(uint32_t), true));
        CK(cudaMallocHost((void **)&r.h_err, sizeof(uint32_t)));
        CK(cudaEventCreateWithFlags(&r.h2d, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&r.comp, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&r.done, cudaEventDisableTiming));
    }
    // the staged form's scratch buffers are shared between batches: one stream
    if (h->mode != EMIDA_GB_MODE_PLAIN && !h->comp_alt)
        CK(cudaStreamCreateWithFlags(&h->comp_alt, cudaStreamNonBlocking));
    h->ring = std::move(ring);
    return EMIDA_GB_OK;
}

int emida_gb_submit(emida_gb_handle *h, const void *batch, uint32_t patterns, uint64_t *ticket)
{
    trace_range tr("emida_gb_submit");
    if (!h || !batch || !ticket) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    if (patterns == 0 || patterns > h->B)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "patterns must be in [1, batch_size]");
    if (!h->ref_set) return fail(EMIDA_GB_INVALID_ARGUMENT, "reference pattern not set");
    std::lock_guard<std::mutex> lk(h->mu);
    CKS(ring_init(h));
    const uint64_t t = h->next_ticket;
    const size_t si = t % h->ring.size();
    auto &r = h->ring[si];
    if (r.busy)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "all %zu slots in flight: wait for ticket %llu first",
                    h->ring.size(), (unsigned long long)r.ticket);
    cudaStream_t cs = h->comp_alt && (t & 1) ? h->comp_alt : h->comp;
    cudaPointerAttributes pa{};
    CK(cudaPointerGetAttributes(&pa, batch));
    // device batches are used in place; pinned host batches are copied or read
    // in place as the ingest mode says
    const bool in_place_host = pa.type == cudaMemoryTypeHost && h->ingest == EMIDA_GB_INGEST_IN_PLACE;
    const bool gather = pa.type == cudaMemoryTypeHost && h->ingest == EMIDA_GB_INGEST_GATHER &&
                        (uintptr_t)batch % 16 == 0;
    const bool sm_copy = pa.type == cudaMemoryTypeHost && h->ingest == EMIDA_GB_INGEST_SM_COPY &&
                         (uintptr_t)batch % 16 == 0;
    const void *src = batch;
    batch_view compact{size2{gather_width(h->slice.x), h->S * h->slice.y}, h->d_begins_compact};
    const batch_view *view = nullptr;
    int grid = 0;
    if (gather) {
        // only the ROI rows cross the host link, packed by a gather kernel on
        // GATHER_CTAS CTAs of the path's footprint; the path launches that
        // many CTAs short of a full wave, so the gather of the next batch runs
        // beside it
        const size_t smem = h->mode == EMIDA_GB_MODE_FUSED ? fused_smem_bytes(h->w2, h->dbl)
                                                           : brute_tc_smem_bytes();
        CK(cudaStreamWaitEvent(h->in_stream, r.comp, 0));
        CK(run_gather_rois(static_cast<const uint16_t *>(batch), h->src, h->d_begins, h->S, h->slice,
                           patterns, static_cast<uint16_t *>(h->d_in[si]), GATHER_CTAS, smem,
                           h->in_stream));
        CK(cudaEventRecord(r.h2d, h->in_stream));
        CK(cudaStreamWaitEvent(cs, r.h2d, 0));
        src = h->d_in[si];
        view = &compact;
        grid = -GATHER_CTAS;
    } else if (sm_copy) {
        // the row bands cross the host link by SM loads on COPY_CTAS CTAs of
        // the path's footprint, beside the previous batch's path, which
        // launches that many CTAs short of a full wave
        const size_t smem = h->mode == EMIDA_GB_MODE_FUSED   ? fused_smem_bytes(h->w2, h->dbl)
                            : h->mode == EMIDA_GB_MODE_TENSOR ? brute_tc_smem_bytes()
                                                              : 0;
        const uint64_t pat16 = (uint64_t)h->src.x * h->src.y * h->in_elem / 16;
        CK(cudaStreamWaitEvent(h->in_stream, r.comp, 0));
        CK(run_copy_bands(batch, h->d_in[si], h->d_band_runs, h->n_band_runs, pat16, patterns, COPY_CTAS,
                          smem, h->in_stream));
        CK(cudaEventRecord(r.h2d, h->in_stream));
        CK(cudaStreamWaitEvent(cs, r.h2d, 0));
        src = h->d_in[si];
        grid = h->mode == EMIDA_GB_MODE_PLAIN ? 0 : -COPY_CTAS;
    } else if (!(pa.type == cudaMemoryTypeDevice || pa.type == cudaMemoryTypeManaged || in_place_host)) {
        // the input buffer is free once the slot's previous computation ran
        CK(cudaStreamWaitEvent(h->in_stream, r.comp, 0));
        CKS(copy_patterns(h, h->d_in[si], batch, patterns, h->in_stream));
        CK(cudaEventRecord(r.h2d, h->in_stream));
        CK(cudaStreamWaitEvent(cs, r.h2d, 0));
        src = h->d_in[si];
    }
    if (h->selftest_budget > 0) {
        // armed by emida_gb_selftest_arm_submit: this batch's error word is set
        // by a bounded wait that runs out, as a real timeout of its path would
        k_selftest_wait<<<1, 32, 0, cs>>>(r.d_err, (long long)h->selftest_budget);
        CK(cudaGetLastError());
        h->selftest_budget = 0;
    }
    // the neighbourhoods are scratch for the staged form only; the fused and
    // tensor forms of two batches may run at once and keep them in shared memory
    CKS(run_any(h, src, patterns, r.d_maxes, h->mode == EMIDA_GB_MODE_PLAIN ? h->d_neigh : nullptr,
                r.d_offsets, r.d_coefs, cs, view, grid, r.d_err));
    CK(cudaEventRecord(r.comp, cs));
    CK(cudaStreamWaitEvent(h->out_stream, r.comp, 0));
    const size_t n = (size_t)patterns * h->S;
    CK(cudaMemcpyAsync(r.h_offsets, r.d_offsets, 2 * sizeof(double) * n, cudaMemcpyDeviceToHost, h->out_stream));
    CK(cudaMemcpyAsync(r.h_coefs, r.d_coefs, 6 * sizeof(double) * n, cudaMemcpyDeviceToHost, h->out_stream));
    CK(cudaMemcpyAsync(r.h_maxes, r.d_maxes, h->di_elem * n, cudaMemcpyDeviceToHost, h->out_stream));
    // the error word travels with the results: wait() reads it without a synchronous copy
    CK(cudaMemcpyAsync(r.h_err, r.d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->out_stream));
    CK(cudaEventRecord(r.done, h->out_stream));
    r.busy = true;
    r.ticket = t;
    r.patterns = patterns;
    h->next_ticket = t + 1;
    *ticket = t;
    return EMIDA_GB_OK;
}

int emida_gb_wait(emida_gb_handle *h, uint64_t ticket, double *offsets, double *coefs,
                  uint32_t *peaks)
{
    trace_range tr("emida_gb_wait");
    if (!h || !offsets) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    emida_gb_handle::slot *r = nullptr;
    {
        std::lock_guard<std::mutex> lk(h->mu);
        if (h->ring.empty()) return fail(EMIDA_GB_INVALID_ARGUMENT, "nothing submitted");
        r = &h->ring[ticket % h->ring.size()];
        if (!r->busy || r->ticket != ticket)
            return fail(EMIDA_GB_INVALID_ARGUMENT, "unknown ticket %llu", (unsigned long long)ticket);
    }
    CK(cudaEventSynchronize(r->done));
    if (const uint32_t flags = *r->h_err) {
        // The batch failed its device check.  Its ticket is consumed and its
        // slot released, with the slot's word cleared (and the clear complete)
        // before the slot can be submitted again.
        *r->h_err = 0;
        cudaError_t e = cudaMemsetAsync(r->d_err, 0, sizeof(uint32_t), h->out_stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->out_stream);
        {
            std::lock_guard<std::mutex> lk(h->mu);
            r->busy = false;
        }
        if (e != cudaSuccess)
            return fail(EMIDA_GB_CUDA_ERROR, "clearing the error word of ticket %llu: %s",
                        (unsigned long long)ticket, cudaGetErrorString(e));
        return device_flags_status(flags);
    }
    const size_t n = (size_t)r->patterns * h->S;
    std::memcpy(offsets, r->h_offsets, 2 * sizeof(double) * n);
    if (coefs) std::memcpy(coefs, r->h_coefs, 6 * sizeof(double) * n);
    if (peaks)
        for (size_t i = 0; i < n; ++i)
            peaks[i] = h->dbl ? reinterpret_cast<const data_index<double> *>(r->h_maxes)[i].index
                              : reinterpret_cast<const data_index<float> *>(r->h_maxes)[i].index;
    std::lock_guard<std::mutex> lk(h->mu);
    r->busy = false;
    return EMIDA_GB_OK;
}

int emida_gb_run_device(emida_gb_handle *h, const void *dev_patterns, uint32_t patterns,
                        double *dev_offsets, double *dev_coefs, void *dev_maxes, void *dev_neigh,
                        void *stream)
{
    trace_range tr("emida_gb_run_device");
    if (!h || !dev_patterns || !dev_offsets) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    if (!h->ref_set) return fail(EMIDA_GB_INVALID_ARGUMENT, "reference pattern not set");
    bool on_device = true;
    CKS(pattern_location(dev_patterns, on_device));  // device or pinned host memory
    cudaStream_t st = stream ? (cudaStream_t)stream : h->comp;
    std::lock_guard<std::mutex> lk(h->mu);
    return run_any(h, dev_patterns, patterns, dev_maxes, dev_neigh, dev_offsets, dev_coefs, st);
}

int emida_gb_time_device(emida_gb_handle *h, const void *dev_patterns, uint32_t patterns,
                         double *dev_offsets, int repeats, float *ms)
{
    if (!h || !ms || repeats < 1) return fail(EMIDA_GB_INVALID_ARGUMENT, "bad argument");
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, h->comp));
    for (int i = 0; i < repeats; ++i)
        CKS(emida_gb_run_device(h, dev_patterns, patterns, dev_offsets, nullptr, nullptr, nullptr, nullptr));
    CK(cudaEventRecord(b, h->comp));
    CK(cudaEventSynchronize(b));
    CK(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return check_device_error(h);
}

int emida_gb_resolved_mode(const emida_gb_handle *h) { return h ? h->mode : -1; }

int emida_gb_ingest(const emida_gb_handle *h) { return h ? h->ingest : -1; }

int emida_gb_set_ingest(emida_gb_handle *h, int mode)
{
    if (!h) return fail(EMIDA_GB_INVALID_ARGUMENT, "null handle");
    if (mode < EMIDA_GB_INGEST_COPY || mode > EMIDA_GB_INGEST_SM_COPY || mode == 2)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "invalid ingest mode %d", mode);
    std::lock_guard<std::mutex> lk(h->mu);
    const bool ok = mode == EMIDA_GB_INGEST_GATHER    ? h->gather_allowed
                    : mode == EMIDA_GB_INGEST_SM_COPY ? h->sm_copy_allowed
                    : mode == EMIDA_GB_INGEST_COPY    ? true
                                                      : h->in_place_allowed;
    h->ingest = ok ? mode : EMIDA_GB_INGEST_COPY;
    return EMIDA_GB_OK;
}
void *emida_gb_stream(emida_gb_handle *h) { return h ? (void *)h->comp : nullptr; }

int emida_gb_streams(emida_gb_handle *h, void **in_stream, void **out_stream)
{
    if (!h) return fail(EMIDA_GB_INVALID_ARGUMENT, "null handle");
    if (in_stream) *in_stream = (void *)h->in_stream;
    if (out_stream) *out_stream = (void *)h->out_stream;
    return EMIDA_GB_OK;
}

int emida_gb_stage_buffers(emida_gb_handle *h, void **pic, void **temp, void **maps)
{
    if (!h) return fail(EMIDA_GB_INVALID_ARGUMENT, "null handle");
    std::lock_guard<std::mutex> lk(h->mu);
    CKS(stage_hooks(h));
    if (pic) *pic = h->hk.pic;
    if (temp) *temp = h->hk.temp;
    if (maps) *maps = h->hk.map;
    return EMIDA_GB_OK;
}

int emida_gb_cross_corr_fft(emida_gb_handle *h)
{
    trace_range tr("emida_gb_cross_corr_fft");
    if (!h) return fail(EMIDA_GB_INVALID_ARGUMENT, "null handle");
    if (!h->fft) return fail(EMIDA_GB_UNSUPPORTED, "cross_corr_fft needs the FFT policy");
    std::lock_guard<std::mutex> lk(h->mu);
    CKS(stage_hooks(h));
    const fft_tables t{h->hk.tw_row, h->hk.tw_col, 2 * h->slice.x, 2 * h->slice.y};
    CK(run_fft_r2c(h->hk.pic, h->hk.spec, h->N, t, h->dbl, h->comp));
    CK(run_hadamard(h->hk.spec, h->hk.temp, t.h2 * (t.w2 / 2 + 1), h->S, h->B, h->dbl, h->comp));
    CK(run_fft_c2r(h->hk.spec, h->hk.map, h->N, t, h->dbl, h->comp));
    CK(cudaStreamSynchronize(h->comp));
    return EMIDA_GB_OK;
}
int emida_gb_launches_per_run(const emida_gb_handle *h)
{
    if (!h) return -1;
    if (h->mode == EMIDA_GB_MODE_FUSED || h->mode == EMIDA_GB_MODE_TENSOR) return 1;
    return h->fft ? 10 : 6;
}

void emida_gb_destroy(emida_gb_handle *h)
{
    if (!h) return;
    if (h->comp) cudaStreamSynchronize(h->comp);
    if (h->comp_alt) cudaStreamSynchronize(h->comp_alt);
    if (h->in_stream) cudaStreamSynchronize(h->in_stream);
    if (h->out_stream) cudaStreamSynchronize(h->out_stream);
    for (auto &r : h->ring) {
        if (r.h_offsets) cudaFreeHost(r.h_offsets);
        if (r.h_coefs) cudaFreeHost(r.h_coefs);
        if (r.h_maxes) cudaFreeHost(r.h_maxes);
        if (r.h_err) cudaFreeHost(r.h_err);
        for (cudaEvent_t e : {r.h2d, r.comp, r.done})
            if (e) cudaEventDestroy(e);
    }
    for (void *p : h->allocs) cudaFree(p);
    for (auto e : h->in_done)
        if (e) cudaEventDestroy(e);
    for (auto e : h->in_used)
        if (e) cudaEventDestroy(e);
    if (h->comp_done) cudaEventDestroy(h->comp_done);
    if (h->out_done) cudaEventDestroy(h->out_done);
    if (h->comp) cudaStreamDestroy(h->comp);
    if (h->comp_alt) cudaStreamDestroy(h->comp_alt);
    if (h->in_stream) cudaStreamDestroy(h->in_stream);
    if (h->out_stream) cudaStreamDestroy(h->out_stream);
    delete h;
}

// ---- memory helpers -----------------------------------------------------------
// ---- deformation fit downstream of the path ----------------------------------
static int check_homography(const double *mids, const double *offsets, uint32_t n_rois,
                            const double *centre, double *out)
{
    if (!mids || !offsets || !centre || !out) return fail(EMIDA_GB_INVALID_ARGUMENT, "null argument");
    if (n_rois < HOMOGRAPHY_MIN_ROIS || n_rois > HOMOGRAPHY_MAX_ROIS)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "the deformation fit takes %u..%u ROIs per pattern (got %u)",
                    HOMOGRAPHY_MIN_ROIS, HOMOGRAPHY_MAX_ROIS, n_rois);
    return EMIDA_GB_OK;
}

int emida_gb_fit_homography(const double *mids, const double *offsets, uint32_t n_rois,
                            uint32_t patterns, const double *centre, const double *coefs,
                            double min_det, double *out, void *stream)
{
    CKS(check_homography(mids, offsets, n_rois, centre, out));
    CK(launch_homography(mids, offsets, n_rois, patterns, centre[0], centre[1], centre[2], coefs, min_det,
                         out, (cudaStream_t)stream));
    return EMIDA_GB_OK;
}

int emida_gb_time_fit_homography(const double *mids, const double *offsets, uint32_t n_rois,
                                 uint32_t patterns, const double *centre, const double *coefs,
                                 double min_det, double *out, int repeats, float *ms)
{
    CKS(check_homography(mids, offsets, n_rois, centre, out));
    if (repeats < 1 || !ms) return fail(EMIDA_GB_INVALID_ARGUMENT, "repeats must be >= 1");
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, 0));
    for (int r = 0; r < repeats; ++r)
        CK(launch_homography(mids, offsets, n_rois, patterns, centre[0], centre[1], centre[2], coefs,
                             min_det, out, 0));
    CK(cudaEventRecord(b, 0));
    CK(cudaEventSynchronize(b));
    CK(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return EMIDA_GB_OK;
}

int emida_gb_set_device(int device)
{
    CK(cudaSetDevice(device));
    return EMIDA_GB_OK;
}

int emida_gb_device_count(int *count)
{
    CK(cudaGetDeviceCount(count));
    return EMIDA_GB_OK;
}
int emida_gb_malloc(void **p, size_t bytes)
{
    CK(cudaMalloc(p, bytes ? bytes : 16));
    return EMIDA_GB_OK;
}
int emida_gb_free(void *p)
{
    CK(cudaFree(p));
    return EMIDA_GB_OK;
}
int emida_gb_memset(void *p, int v, size_t bytes)
{
    CK(cudaMemset(p, v, bytes));
    return EMIDA_GB_OK;
}
int emida_gb_memcpy_h2d(void *d, const void *s, size_t bytes)
{
    CK(cudaMemcpy(d, s, bytes, cudaMemcpyHostToDevice));
    return EMIDA_GB_OK;
}
int emida_gb_memcpy_d2d(void *d, const void *s, size_t bytes)
{
    CK(cudaMemcpy(d, s, bytes, cudaMemcpyDeviceToDevice));
    return EMIDA_GB_OK;
}
int emida_gb_memcpy_d2h(void *d, const void *s, size_t bytes)
{
    CK(cudaMemcpy(d, s, bytes, cudaMemcpyDeviceToHost));
    return EMIDA_GB_OK;
}
int emida_gb_malloc_host(void **p, size_t bytes)
{
    CK(cudaMallocHost(p, bytes ? bytes : 16));
    return EMIDA_GB_OK;
}
int emida_gb_free_host(void *p)
{
    CK(cudaFreeHost(p));
    return EMIDA_GB_OK;
}
int emida_gb_synchronize(void)
{
    CK(cudaDeviceSynchronize());
    return EMIDA_GB_OK;
}

}  // extern "C"

extern "C" {

int emida_gb_selftest_bounded_wait(emida_gb_handle *h, int64_t budget_cycles)
{
    if (!h) return fail(EMIDA_GB_INVALID_ARGUMENT, "null handle");
    if (budget_cycles < 1 || budget_cycles > 4000000000LL)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "budget must be in [1, 4e9] cycles");
    std::lock_guard<std::mutex> lk(h->mu);
    k_selftest_wait<<<1, 32, 0, h->comp>>>(h->d_err, (long long)budget_cycles);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->comp));
    return check_device_error(h);
}

int emida_gb_selftest_arm_submit(emida_gb_handle *h, int64_t budget_cycles)
{
    if (!h) return fail(EMIDA_GB_INVALID_ARGUMENT, "null handle");
    if (budget_cycles < 1 || budget_cycles > 4000000000LL)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "budget must be in [1, 4e9] cycles");
    std::lock_guard<std::mutex> lk(h->mu);
    h->selftest_budget = budget_cycles;
    return EMIDA_GB_OK;
}

// ---- per-stage launchers --------------------------------------------------------
int emida_gb_run_sum(const void *pics, int in_type, uint32_t src_w, uint32_t src_h,
                     const uint32_t *dev_begins, uint32_t n_rois, uint32_t slice_w,
                     uint32_t slice_h, uint32_t batch, void *sums)
{
    CK(run_sums(pics, in_type, size2{src_w, src_h}, reinterpret_cast<const uint2 *>(dev_begins),
                n_rois, size2{slice_w, slice_h}, batch, sums, 0));
    CK(cudaDeviceSynchronize());
    return EMIDA_GB_OK;
}

int emida_gb_run_prepare(const void *pics, int in_type, int precision, void *slices,
                         const void *hann, const void *sums, const uint32_t *dev_begins,
                         uint32_t src_w, uint32_t src_h, uint32_t slice_w, uint32_t slice_h,
                         uint32_t out_w, uint32_t out_h, uint32_t n_rois, uint32_t batch)
{
    CK(run_prepare(pics, in_type, precision == EMIDA_GB_DOUBLE, slices, hann, sums,
                   reinterpret_cast<const uint2 *>(dev_begins), size2{src_w, src_h},
                   size2{slice_w, slice_h}, size2{out_w, out_h}, n_rois, batch, 0));
    CK(cudaDeviceSynchronize());
    return EMIDA_GB_OK;
}

int emida_gb_run_cross_corr(const void *pics, const void *ref, void *res, int precision,
                            uint32_t w, uint32_t h, uint32_t res_w, uint32_t res_h,
                            uint32_t ref_slices, uint32_t batch)
{
    CK(run_cross_corr(pics, ref, res, precision == EMIDA_GB_DOUBLE, size2{w, h},
                      size2{res_w, res_h}, ref_slices, batch, 0));
    CK(cudaDeviceSynchronize());
    return EMIDA_GB_OK;
}

static int stage_tables(int precision, uint32_t w2, uint32_t h2, emida_gb_handle &tmp, fft_tables &t)
{
    tmp.dbl = precision == EMIDA_GB_DOUBLE;
    CKS(upload_twiddles(&tmp, &tmp.d_tw_row, w2));
    CKS(upload_twiddles(&tmp, &tmp.d_tw_col, h2));
    t = fft_tables{tmp.d_tw_row, tmp.d_tw_col, w2, h2};
    return EMIDA_GB_OK;
}

int emida_gb_run_fft_r2c(const void *real_in, void *spec, uint32_t maps, uint32_t w2,
                         uint32_t h2, int precision)
{
    emida_gb_handle tmp;
    fft_tables t;
    int st = stage_tables(precision, w2, h2, tmp, t);
    if (st == EMIDA_GB_OK) {
        cudaError_t e = run_fft_r2c(real_in, spec, maps, t, precision == EMIDA_GB_DOUBLE, 0);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) st = fail(EMIDA_GB_CUDA_ERROR, "fft r2c: %s", cudaGetErrorString(e));
    }
    for (void *p : tmp.allocs) cudaFree(p);
    tmp.allocs.clear();
    return st;
}

int emida_gb_run_fft_c2r(void *spec, void *real_out, uint32_t maps, uint32_t w2, uint32_t h2,
                         int precision)
{
    emida_gb_handle tmp;
    fft_tables t;
    int st = stage_tables(precision, w2, h2, tmp, t);
    if (st == EMIDA_GB_OK) {
        cudaError_t e = run_fft_c2r(spec, real_out, maps, t, precision == EMIDA_GB_DOUBLE, 0);
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
        if (e != cudaSuccess) st = fail(EMIDA_GB_CUDA_ERROR, "fft c2r: %s", cudaGetErrorString(e));
    }
    for (void *p : tmp.allocs) cudaFree(p);
    tmp.allocs.clear();
    return st;
}

}  // extern "C"

// ---- allocation-free forward FFT --------------------------------------------------
// emida_gb_run_fft_r2c builds its two twiddle tables in cudaMalloc'd memory and
// frees them on return.  The variant below keeps them in one fixed device array
// instead: the row table at byte 0, the column table at byte NOALLOC_COL_OFFSET,
// each up to NOALLOC_MAX_SIDE complex doubles, 32 KiB in all.  It runs on a
// non-blocking stream of its own, so it neither waits for nor holds up the work
// of any other stream on the device.
namespace {

constexpr uint32_t NOALLOC_MAX_SIDE = 1024;
constexpr size_t NOALLOC_COL_OFFSET = NOALLOC_MAX_SIDE * sizeof(double2);
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) unsigned char g_noalloc_twiddles[2 * NOALLOC_COL_OFFSET];

// Per device: the array's device address and the entry point's stream.
struct noalloc_device {
    void *scratch = nullptr;
    cudaStream_t stream = nullptr;
};
std::mutex g_noalloc_mutex;
noalloc_device g_noalloc[NOALLOC_MAX_DEVICES];

// The current device's set-up, done by the first call made with that device
// current and cached afterwards: the address of g_noalloc_twiddles (a host-side
// name that no kernel may be given) and a non-blocking stream.
int noalloc_setup(noalloc_device *out)
{
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return fail(EMIDA_GB_UNSUPPORTED, "fft r2c (no-alloc): device %d beyond the %d supported",
                    dev, NOALLOC_MAX_DEVICES);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    noalloc_device &d = g_noalloc[dev];
    if (!d.scratch) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_twiddles);
        if (e != cudaSuccess || !p)
            return fail(EMIDA_GB_CUDA_ERROR, "fft r2c (no-alloc): scratch address on device %d: %s",
                        dev, cudaGetErrorString(e));
        cudaStream_t st = nullptr;
        e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e != cudaSuccess)
            return fail(EMIDA_GB_CUDA_ERROR, "fft r2c (no-alloc): stream on device %d: %s", dev,
                        cudaGetErrorString(e));
        d.stream = st;
        d.scratch = p;
    }
    *out = d;
    return EMIDA_GB_OK;
}

// The same values emida_gb::host::upload_twiddles computes, written into a
// caller-provided host array.
template <typename C> void twiddles_into(C *w, uint32_t n)
{
    const double PI = 3.14159265358979323846;
    for (uint32_t j = 0; j < n; ++j) {
        if constexpr (sizeof(C) == sizeof(double2))
            w[j] = make_double2(std::cos(2 * PI * j / n), -std::sin(2 * PI * j / n));
        else
            w[j] = make_float2((float)std::cos(2 * PI * j / n), (float)-std::sin(2 * PI * j / n));
    }
}

template <typename C>
int fft_r2c_noalloc(const void *real_in, void *spec, uint32_t maps, uint32_t w2, uint32_t h2,
                    const noalloc_device &d)
{
    // Host staging on the stack: two tables of at most NOALLOC_MAX_SIDE entries.
    // The copies from pageable memory have read them before they return.
    C row[NOALLOC_MAX_SIDE], col[NOALLOC_MAX_SIDE];
    twiddles_into(row, w2);
    twiddles_into(col, h2);
    auto *scratch = static_cast<unsigned char *>(d.scratch);
    CK(cudaMemcpyAsync(scratch, row, w2 * sizeof(C), cudaMemcpyHostToDevice, d.stream));
    CK(cudaMemcpyAsync(scratch + NOALLOC_COL_OFFSET, col, h2 * sizeof(C), cudaMemcpyHostToDevice,
                       d.stream));
    const fft_tables t{scratch, scratch + NOALLOC_COL_OFFSET, w2, h2};
    CK(run_fft_r2c(real_in, spec, maps, t, sizeof(C) == sizeof(double2), d.stream));
    CK(cudaStreamSynchronize(d.stream));
    return EMIDA_GB_OK;
}

}  // namespace

extern "C" {

int emida_gb_run_fft_r2c_noalloc(const void *real_in, void *spec, uint32_t maps, uint32_t w2,
                                 uint32_t h2, int precision)
{
    if (precision != EMIDA_GB_DOUBLE && precision != EMIDA_GB_FLOAT)
        return fail(EMIDA_GB_INVALID_ARGUMENT, "fft r2c (no-alloc): unknown precision %d", precision);
    if (w2 == 0 || h2 == 0 || w2 > NOALLOC_MAX_SIDE || h2 > NOALLOC_MAX_SIDE)
        return fail(EMIDA_GB_INVALID_ARGUMENT,
                    "fft r2c (no-alloc): transform %u x %u outside 1..%u per side (the fixed "
                    "twiddle scratch holds %u entries per table)",
                    w2, h2, NOALLOC_MAX_SIDE, NOALLOC_MAX_SIDE);
    if (maps == 0) return EMIDA_GB_OK;
    if (!real_in || !spec) return fail(EMIDA_GB_INVALID_ARGUMENT, "fft r2c (no-alloc): null buffer");
    noalloc_device d;
    CKS(noalloc_setup(&d));
    return precision == EMIDA_GB_DOUBLE ? fft_r2c_noalloc<double2>(real_in, spec, maps, w2, h2, d)
                                        : fft_r2c_noalloc<float2>(real_in, spec, maps, w2, h2, d);
}

int emida_gb_run_hadamard(void *pics, const void *ref, uint32_t one_area, uint32_t ref_slices,
                          uint32_t batch, int precision)
{
    CK(run_hadamard(pics, ref, one_area, ref_slices, batch, precision == EMIDA_GB_DOUBLE, 0));
    CK(cudaDeviceSynchronize());
    return EMIDA_GB_OK;
}

int emida_gb_run_maxarg(const void *maps, uint32_t map_size, uint32_t n, void *maxes, int precision)
{
    CK(run_maxarg(maps, map_size, n, maxes, precision == EMIDA_GB_DOUBLE, 0));
    CK(cudaDeviceSynchronize());
    return EMIDA_GB_OK;
}

int emida_gb_run_extract_neighbors(const void *maps, const void *maxes, void *neigh, int s,
                                   uint32_t cross_w, uint32_t cross_h, uint32_t n, int policy,
                                   int precision)
{
    CK(run_extract_neighbors(maps, maxes, neigh, s, size2{cross_w, cross_h}, n, policy,
                             precision == EMIDA_GB_DOUBLE, 0));
    CK(cudaDeviceSynchronize());
    return EMIDA_GB_OK;
}

}  // extern "C"
