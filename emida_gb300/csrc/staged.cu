// staged.cu -- the plain staged form: one kernel per stage of the reference's
// get_offset_core (src/gpu_offset.hpp:234-278), each stage reading and writing
// HBM buffers laid out as the reference lays them out.  It is the baseline the
// fused kernel is measured against and the path for every size the fused kernel
// does not cover (any ROI size, brute policy, odd FFT lengths).
#include <algorithm>

#include "device_fit.cuh"
#include "fft.cuh"
#include "staged.cuh"

namespace emida_gb {

namespace {

constexpr int BLOCK = 256;

template <typename T> struct sum_of { using type = double; };
template <> struct sum_of<uint16_t> { using type = uint32_t; };

template <typename V>
__device__ __forceinline__ V block_sum(V v, V *scratch)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) scratch[warp] = v;
    __syncthreads();
    V total = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) total += scratch[w];
    return total;
}

// ---- sums (src/sum.cu:109-158) ----------------------------------------------
template <typename IN>
__global__ void __launch_bounds__(BLOCK) k_sums(const IN *__restrict__ pics, size2 src,
                                                const uint2 *__restrict__ begins, uint32_t n_rois,
                                                size2 slice, typename sum_of<IN>::type *sums,
                                                const void *const *__restrict__ ptrs)
{
    using S = typename sum_of<IN>::type;
    __shared__ S scratch[32];
    const uint32_t pair = blockIdx.x, pic = pair / n_rois, roi = pair % n_rois;
    const uint2 b = begins[roi];
    const IN *base = ptrs ? reinterpret_cast<const IN *>(ptrs[pic]) : pics + (size_t)pic * src.x * src.y;
    const IN *p = base + (size_t)b.y * src.x + b.x;
    S acc = 0;
    const uint32_t area = slice.x * slice.y;
    for (uint32_t i = threadIdx.x; i < area; i += BLOCK)
        acc += (S)p[(size_t)(i / slice.x) * src.x + (i % slice.x)];
    S total = block_sum(acc, scratch);
    if (threadIdx.x == 0) sums[pair] = total;
}

// ---- prepare (src/prepare_pics.cu:11-42) -----------------------------------
template <typename IN, typename T>
__global__ void __launch_bounds__(BLOCK)
    k_prepare(const IN *__restrict__ pics, T *__restrict__ out, const T *__restrict__ hann,
              const typename sum_of<IN>::type *__restrict__ sums,
              const uint2 *__restrict__ begins, size2 src, size2 slice, size2 out_size,
              uint32_t n_rois, uint32_t n_pairs, const void *const *__restrict__ ptrs)
{
    const uint64_t tid = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    const uint32_t area = slice.x * slice.y;
    const uint64_t pair = tid / area;
    if (pair >= n_pairs) return;
    const uint32_t within = (uint32_t)(tid % area), x = within % slice.x, y = within / slice.x;
    const uint32_t pic = (uint32_t)(pair / n_rois), roi = (uint32_t)(pair % n_rois);
    const uint2 b = begins[roi];
    const IN *base = ptrs ? reinterpret_cast<const IN *>(ptrs[pic]) : pics + (size_t)pic * src.x * src.y;
    T pixel = (T)base[(size_t)(b.y + y) * src.x + b.x + x];
    pixel -= (T)sums[pair] / (T)area;
    pixel = pixel * hann[x] * hann[slice.x + y];
    out[pair * out_size.x * out_size.y + (size_t)y * out_size.x + x] = pixel;
}

// ---- brute-force correlation (src/cross_corr.cu:11-66) ----------------------
// One block per (lag row, pair); both ROIs staged in shared memory.
template <typename T> __device__ __forceinline__ T mul_rn(T a, T b);
template <> __device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
template <typename T> __device__ __forceinline__ T add_rn(T a, T b);
template <> __device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

template <typename T>
__global__ void __launch_bounds__(BLOCK)
    k_cross_corr(const T *__restrict__ pics, const T *__restrict__ ref, T *__restrict__ res,
                 size2 size, size2 res_size, uint32_t ref_slices, uint32_t pair0)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *sp = reinterpret_cast<T *>(smem_raw);
    T *sr = sp + size.x * size.y;
    // pairs run in launches of at most 65,535 (grid.y); pair0 is the launch's first
    const uint32_t py = blockIdx.x, pair = pair0 + blockIdx.y;
    const uint32_t area = size.x * size.y;
    const T *p = pics + (size_t)pair * area;
    const T *r = ref + (size_t)(pair % ref_slices) * area;
    for (uint32_t i = threadIdx.x; i < area; i += BLOCK) {
        sp[i] = p[i];
        sr[i] = r[i];
    }
    __syncthreads();
    const int rx = (int)(res_size.x - 1) / 2, ry = (int)(res_size.y - 1) / 2;
    const int sy = (int)py - ry;
    const int y_beg = sy < 0 ? -sy : 0;
    const int y_end = (int)size.y - sy < (int)size.y ? (int)size.y - sy : (int)size.y;
    for (uint32_t px = threadIdx.x; px < res_size.x; px += BLOCK) {
        const int sx = (int)px - rx;
        const int x_beg = sx < 0 ? -sx : 0;
        const int x_end = (int)size.x - sx < (int)size.x ? (int)size.x - sx : (int)size.x;
        T sum = 0;
        for (int y = y_beg; y < y_end; ++y)
            for (int x = x_beg; x < x_end; ++x)
                sum = add_rn(sum, mul_rn(sp[(y + sy) * (int)size.x + x + sx], sr[y * (int)size.x + x]));
        res[(size_t)pair * res_size.x * res_size.y + (size_t)py * res_size.x + px] = sum;
    }
}

// ---- generic mixed-radix Stockham FFT over lines -----------------------------
enum line_mode { LM_R2C_ROWS = 0, LM_C2C_COLS = 1, LM_C2R_ROWS = 2 };

struct line_plan {
    int n;            // transform length
    int npass;
    int radix[24];
};

static line_plan make_plan(int n)
{
    line_plan p{};
    p.n = n;
    int m = n;
    while (m % 4 == 0) { p.radix[p.npass++] = 4; m /= 4; }
    while (m % 2 == 0) { p.radix[p.npass++] = 2; m /= 2; }
    for (int f = 3; m > 1; f += 2)
        while (m % f == 0) { p.radix[p.npass++] = f; m /= f; }
    return p;
}

template <typename C>
__device__ __forceinline__ C tw_get(const C *tw, int j, int dir)
{
    C w = tw[j];
    return dir > 0 ? cconj(w) : w;
}

template <typename T>
__global__ void __launch_bounds__(BLOCK)
    k_fft_lines(const void *in, void *out, int mode, int dir, line_plan plan, uint32_t n_lines,
                uint32_t lines_per_map, uint32_t half, uint32_t map_len_in, uint32_t map_len_out,
                const cplx<T> *__restrict__ twg, int lpb)
{
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = plan.n;
    C *tw = reinterpret_cast<C *>(smem_raw);
    C *buf = tw + n;
    for (int i = threadIdx.x; i < n; i += BLOCK) tw[i] = twg[i];
    const int tpl = BLOCK / lpb, l = threadIdx.x / tpl, lt = threadIdx.x % tpl;
    const uint32_t line = blockIdx.x * lpb + l;
    const bool live = l < lpb && line < n_lines;
    // rows of up to 32 threads a line stay inside one warp between passes
    const bool warp_lines = mode != LM_C2C_COLS && tpl <= 32;
    C *b0 = buf + (size_t)l * 2 * n, *b1 = b0 + n;
    const uint32_t map = live ? line / lines_per_map : 0, li = live ? line % lines_per_map : 0;

    if (mode == LM_C2C_COLS) {
        // Columns: the block's lpb consecutive columns are loaded row by row by
        // all its threads, so consecutive threads read consecutive columns.
        for (int i = threadIdx.x; i < lpb * n; i += BLOCK) {
            const int l2 = i % lpb, e = i / lpb;
            const uint32_t line2 = blockIdx.x * lpb + l2;
            if (line2 >= n_lines) continue;
            const C *src = reinterpret_cast<const C *>(in) + (size_t)(line2 / lines_per_map) * map_len_in +
                           line2 % lines_per_map;
            buf[(size_t)l2 * 2 * n + e] = src[(size_t)e * half];
        }
    } else if (live) {
        if (mode == LM_R2C_ROWS) {
            const T *src = reinterpret_cast<const T *>(in) + (size_t)map * map_len_in + (size_t)li * n;
            for (int e = lt; e < n; e += tpl) b0[e] = cmake<C>(src[e], (T)0);
        } else {
            const C *src = reinterpret_cast<const C *>(in) + (size_t)map * map_len_in + (size_t)li * half;
            for (int e = lt; e < n; e += tpl)
                b0[e] = (e < (int)half) ? src[e] : cconj(src[n - e]);
        }
    }
    __syncthreads();
    C *cur = b0, *nxt = b1;
    int m = 1;
    for (int ps = 0; ps < plan.npass; ++ps) {
        const int R = plan.radix[ps], nr = n / R, step = n / (m * R);
        if (l < lpb) {
            for (int i = lt; i < nr; i += tpl) {
                const int k = i % m, jj = i / m;
                const int ob = jj * R * m + k;
                if (R == 4) {
                    C a0 = cur[i];
                    C a1 = cmul(cur[i + nr], tw_get(tw, (1 * k * step) % n, dir));
                    C a2 = cmul(cur[i + 2 * nr], tw_get(tw, (2 * k * step) % n, dir));
                    C a3 = cmul(cur[i + 3 * nr], tw_get(tw, (3 * k * step) % n, dir));
                    C s02 = cadd(a0, a2), d02 = csub(a0, a2), s13 = cadd(a1, a3), d13 = csub(a1, a3);
                    // d13 * (-i) forward, * (+i) inverse
                    C r13 = dir < 0 ? cmake<C>(d13.y, -d13.x) : cmake<C>(-d13.y, d13.x);
                    nxt[ob] = cadd(s02, s13);
                    nxt[ob + m] = cadd(d02, r13);
                    nxt[ob + 2 * m] = csub(s02, s13);
                    nxt[ob + 3 * m] = csub(d02, r13);
                } else if (R == 2) {
                    C a0 = cur[i];
                    C a1 = cmul(cur[i + nr], tw_get(tw, (k * step) % n, dir));
                    nxt[ob] = cadd(a0, a1);
                    nxt[ob + m] = csub(a0, a1);
                } else {
                    for (int r = 0; r < R; ++r) {
                        C acc = cmake<C>((T)0, (T)0);
                        for (int q = 0; q < R; ++q) {
                            const int j = (int)(((long long)q * k * step + (long long)nr * ((q * r) % R)) % n);
                            acc = cadd(acc, cmul(cur[i + q * nr], tw_get(tw, j, dir)));
                        }
                        nxt[ob + r * m] = acc;
                    }
                }
            }
        }
        if (warp_lines)
            __syncwarp();
        else
            __syncthreads();
        C *tmp = cur;
        cur = nxt;
        nxt = tmp;
        m *= R;
    }
    if (mode == LM_C2C_COLS) {
        // stored row by row across the block's columns, as they were loaded
        const size_t res = (size_t)(cur - b0);  // n or 0: the pass count's parity
        for (int i = threadIdx.x; i < lpb * n; i += BLOCK) {
            const int l2 = i % lpb, e = i / lpb;
            const uint32_t line2 = blockIdx.x * lpb + l2;
            if (line2 >= n_lines) continue;
            C *dst = reinterpret_cast<C *>(out) + (size_t)(line2 / lines_per_map) * map_len_out +
                     line2 % lines_per_map;
            dst[(size_t)e * half] = buf[(size_t)l2 * 2 * n + res + e];
        }
    } else if (live) {
        if (mode == LM_R2C_ROWS) {
            C *dst = reinterpret_cast<C *>(out) + (size_t)map * map_len_out + (size_t)li * half;
            for (int e = lt; e < (int)half; e += tpl) dst[e] = cur[e];
        } else {
            T *dst = reinterpret_cast<T *>(out) + (size_t)map * map_len_out + (size_t)li * n;
            for (int e = lt; e < n; e += tpl) dst[e] = cur[e].x;
        }
    }
}

template <typename T>
cudaError_t launch_lines(const void *in, void *out, int mode, int dir, int n, uint32_t n_lines,
                         uint32_t lines_per_map, uint32_t half, uint32_t map_len_in,
                         uint32_t map_len_out, const void *tw, cudaStream_t st)
{
    using C = cplx<T>;
    line_plan plan = make_plan(n);
    // rows: n/4 threads a line, one per radix-4 butterfly (a warp per
    // 128-point row)
    int lpb = n >= 1024 ? 1 : 1024 / n;
    if (mode == LM_C2C_COLS) {
        lpb = n >= 512 ? 1 : 512 / n;
        // more columns per block make each row of the block's loads and stores
        // a longer contiguous run: up to 32, in at most 96 KB of shared memory
        const int fit = (int)(((96 * 1024) / sizeof(C) - (size_t)n) / (2 * (size_t)n));
        int want = 32;
        while (want > 1 && want > fit) want >>= 1;
        if (want > lpb) lpb = want;
    }
    if (lpb > BLOCK) lpb = BLOCK;
    while (BLOCK % lpb) --lpb;
    const size_t smem = sizeof(C) * ((size_t)n + 2 * (size_t)n * lpb);
    auto k = k_fft_lines<T>;
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
    }
    const uint32_t grid = (n_lines + lpb - 1) / lpb;
    k<<<grid, BLOCK, smem, st>>>(in, out, mode, dir, plan, n_lines, lines_per_map, half,
                                 map_len_in, map_len_out, reinterpret_cast<const C *>(tw), lpb);
    return cudaGetLastError();
}

// ---- hadamard (src/hadamard.cu:26-41) ---------------------------------------
template <typename T>
__global__ void __launch_bounds__(BLOCK) k_hadamard(cplx<T> *pics, const cplx<T> *__restrict__ ref,
                                                    uint64_t ref_elems, uint64_t total)
{
    const uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    if (i >= total) return;
    pics[i] = cmulc(pics[i], ref[i % ref_elems]);
}

// ---- maxarg (src/maxarg.cu:118-177), first maximum ----------------------------
template <typename T>
__global__ void __launch_bounds__(BLOCK) k_maxarg(const T *__restrict__ maps, uint32_t map_size,
                                                  data_index<T> *out)
{
    __shared__ T sv[32];
    __shared__ uint32_t si[32];
    const T *m = maps + (size_t)blockIdx.x * map_size;
    T bv = m[0];
    uint32_t bi = 0;
    for (uint32_t i = threadIdx.x; i < map_size; i += BLOCK) {
        T v = m[i];
        if (v > bv || (v == bv && i < bi)) {
            bv = v;
            bi = i;
        }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        T ov = __shfl_xor_sync(0xffffffffu, bv, o);
        uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) {
            bv = ov;
            bi = oi;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        sv[warp] = bv;
        si[warp] = bi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        bv = sv[0];
        bi = si[0];
        for (int w = 1; w < BLOCK / 32; ++w)
            if (sv[w] > bv || (sv[w] == bv && si[w] < bi)) {
                bv = sv[w];
                bi = si[w];
            }
        out[blockIdx.x].data = bv;
        out[blockIdx.x].index = bi;
    }
}

// ---- extract_neighbors (src/extract_neighbors.cu:12-41) ----------------------
template <typename T>
__global__ void __launch_bounds__(BLOCK)
    k_extract(const T *__restrict__ maps, const data_index<T> *__restrict__ mi, T *neigh, int s,
              size2 cross, uint32_t n, int policy)
{
    const uint64_t tid = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    const uint32_t s2 = (uint32_t)(s * s);
    if (tid >= (uint64_t)n * s2) return;
    const uint32_t k = (uint32_t)(tid / s2), l = (uint32_t)(tid % s2);
    const uint64_t map_size = policy == POLICY_BRUTE ? (uint64_t)cross.x * cross.y
                                                     : (uint64_t)(cross.x + 1) * (cross.y + 1);
    uint32_t mx, my, x, y;
    shift_pos(mi[k].index, policy, cross.x, cross.y, mx, my);
    neighbour_pos(mx, my, (int)(l % s), (int)(l / s), s, cross.x, cross.y, x, y);
    const uint64_t at = (uint64_t)k * map_size + policy_index(policy, x, y, cross.x, cross.y);
    neigh[tid] = at < (uint64_t)n * map_size ? maps[at] : (T)0;
}

// ---- FP64 fit + finalisation (subpixel_max.hpp:76-97, gpu_offset.hpp:289-298)
template <typename T>
__global__ void __launch_bounds__(BLOCK)
    k_fit(const T *__restrict__ neigh, const data_index<T> *__restrict__ mi, uint32_t n, int s,
          size2 cross, int policy, const double *__restrict__ lstsq, double *offsets,
          double *coefs, const uint32_t *__restrict__ out_base, uint32_t n_rois,
          data_index<T> *maxes_out)
{
    const uint64_t tid = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    if (tid >= n) return;
    const int s2 = s * s;
    double v[81];
    for (int k = 0; k < s2; ++k) v[k] = (double)neigh[tid * s2 + k];
    double c[6];
    for (int j = 0; j < 6; ++j) c[j] = fit_coef(lstsq, v, s, j);
    uint32_t mx, my;
    shift_pos(mi[tid].index, policy, cross.x, cross.y, mx, my);
    double ox, oy;
    fit_offsets(c, mx, my, cross.x, cross.y, s, ox, oy);
    const uint64_t o = out_base ? (uint64_t)out_base[tid / n_rois] + tid % n_rois : tid;
    offsets[2 * o] = ox;
    offsets[2 * o + 1] = oy;
    if (coefs)
        for (int j = 0; j < 6; ++j) coefs[6 * o + j] = c[j];
    if (maxes_out) maxes_out[o] = mi[tid];
}

template <typename T>
__global__ void __launch_bounds__(BLOCK) k_to_colmajor(const cplx<T> *__restrict__ in, cplx<T> *out,
                                                       uint32_t half, uint32_t h2, uint64_t total)
{
    const uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    if (i >= total) return;
    const uint64_t per = (uint64_t)half * h2;
    const uint64_t map = i / per, r = i % per;
    const uint32_t ky = (uint32_t)(r / half), kx = (uint32_t)(r % half);
    out[map * per + (uint64_t)kx * h2 + ky] = in[i];
}

// Column 0 of a column-major reference spectrum, replaced by the spatial
// sequences the fused kernel correlates directly for its packed DC and Nyquist
// slot: entry y of ROI m = (sum_x p[y][x], sum_x (-1)^x p[y][x]) of the
// prepared n x n reference ROI (zero-padded rows give zeros), summed in FP64
// by one warp per row.
template <typename T>
__global__ void __launch_bounds__(BLOCK) k_ref_row_sums(const T *__restrict__ prep, cplx<T> *spec_cm,
                                                        uint32_t n, uint64_t per_map, uint64_t rows)
{
    const uint64_t r = ((uint64_t)blockIdx.x * BLOCK + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= rows) return;  // whole warps leave together
    const uint64_t map = r / n, y = r % n;
    const T *row = prep + r * n;
    double s0 = 0, s1 = 0;
    for (uint32_t x = lane; x < n; x += 32) {
        const double v = (double)row[x];
        s0 += v;
        s1 += (x & 1) ? -v : v;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if (lane == 0) {
        cplx<T> out;
        out.x = (T)s0;
        out.y = (T)s1;
        spec_cm[map * per_map + y] = out;
    }
}

// One thread per ROI row: the 16-byte chunks of the source row that hold the
// row's pixels (CH at most), all loads issued before the stores, so that a
// row costs one round trip (over the host link a read takes microseconds).
template <int CH>
__global__ void __launch_bounds__(256) k_gather_rois(const uint16_t *__restrict__ pics, size2 src,
                                                     const uint2 *__restrict__ begins, uint32_t n_rois,
                                                     size2 slice, uint32_t cw, uint32_t rows,
                                                     uint16_t *__restrict__ out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < rows; i += gridDim.x * blockDim.x) {
        const uint32_t pr = i / slice.y, y = i - pr * slice.y;
        const uint32_t p = pr / n_rois;
        const uint2 b = begins[pr - p * n_rois];
        // chunks [x & ~7, roundup(x + side, 8)) stay inside the row: src.x % 8 == 0
        const uint32_t chunks = ((b.x & 7u) + slice.x + 7) / 8;
        const int4 *s = reinterpret_cast<const int4 *>(
            pics + ((size_t)p * src.y + b.y + y) * src.x + (b.x & ~7u));
        int4 *d = reinterpret_cast<int4 *>(out + (size_t)i * cw);
        int4 v[CH];
#pragma unroll
        for (uint32_t k = 0; k < CH; ++k)
            if (k < chunks) v[k] = s[k];
#pragma unroll
        for (uint32_t k = 0; k < CH; ++k)
            if (k < chunks) d[k] = v[k];
    }
}

// One CTA per (pattern, band) run at a time: the run's 16-byte chunks in
// strides of the block, four loads in flight per thread before their stores,
// so that a CTA keeps 32 KB of host reads in flight over the link.
constexpr int COPY_THREADS = 512;

__global__ void __launch_bounds__(COPY_THREADS)
    k_copy_bands(const int4 *__restrict__ src, int4 *__restrict__ dst, const uint2 *__restrict__ runs,
                 uint32_t n_runs, uint64_t pat16, uint32_t units)
{
    for (uint32_t u = blockIdx.x; u < units; u += gridDim.x) {
        const uint32_t p = u / n_runs;
        const uint2 r = runs[u - p * n_runs];  // (first chunk, chunks) within a pattern
        const uint64_t base = (uint64_t)p * pat16 + r.x;
        const int4 *s = src + base;
        int4 *d = dst + base;
        const uint32_t n = r.y, stride = COPY_THREADS;
        uint32_t i = threadIdx.x;
        for (; i + 3 * stride < n; i += 4 * stride) {
            const int4 a = s[i], b = s[i + stride], c = s[i + 2 * stride], e = s[i + 3 * stride];
            d[i] = a;
            d[i + stride] = b;
            d[i + 2 * stride] = c;
            d[i + 3 * stride] = e;
        }
        for (; i < n; i += stride) d[i] = s[i];
    }
}

inline uint32_t grid_for(uint64_t n) { return (uint32_t)((n + BLOCK - 1) / BLOCK); }

// the largest grid.y a launch takes
constexpr uint32_t CROSS_CORR_MAX_Y = 65535;

}  // namespace

uint32_t gather_width(uint32_t side) { return (side + 14) & ~7u; }

cudaError_t run_gather_rois(const uint16_t *pics, size2 src, const uint2 *begins, uint32_t n_rois,
                            size2 slice, uint32_t patterns, uint16_t *out, int ctas, size_t smem,
                            cudaStream_t st)
{
    if (src.x % 8 || (uintptr_t)pics % 16 || (uintptr_t)out % 16) return cudaErrorInvalidValue;
    const uint32_t cw = gather_width(slice.x), ch = cw / 8;
    if (ch > 17) return cudaErrorInvalidValue;  // ROI sides up to 128
    const size_t pat_out = (size_t)n_rois * slice.y * cw;
    // launches of at most 2^31 rows, so that row indices stay 32-bit
    const uint32_t per = (uint32_t)std::max<uint64_t>(1, (1u << 31) / ((uint64_t)n_rois * slice.y));
    for (uint32_t p0 = 0; p0 < patterns; p0 += per) {
        const uint32_t np = std::min(per, patterns - p0);
        const uint32_t rows = np * n_rois * slice.y;
        if (rows == 0) return cudaSuccess;
        const uint32_t grid = std::min<uint32_t>((rows + 255) / 256, (uint32_t)ctas);
        const uint16_t *in = pics + (size_t)p0 * src.x * src.y;
        uint16_t *o = out + p0 * pat_out;
        auto k = ch <= 4 ? k_gather_rois<4> : ch <= 9 ? k_gather_rois<9> : k_gather_rois<17>;
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<grid, 256, smem, st>>>(in, src, begins, n_rois, slice, cw, rows, o);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t run_copy_bands(const void *src, void *dst, const uint2 *runs, uint32_t n_runs,
                           uint64_t pat16, uint32_t patterns, int ctas, size_t smem,
                           cudaStream_t st)
{
    if ((uintptr_t)src % 16 || (uintptr_t)dst % 16) return cudaErrorInvalidValue;
    const uint64_t units = (uint64_t)patterns * n_runs;
    if (units == 0) return cudaSuccess;
    if (units > 0xffffffffu) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k_copy_bands, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const uint32_t grid = (uint32_t)std::min<uint64_t>(units, (uint64_t)std::max(ctas, 1));
    k_copy_bands<<<grid, COPY_THREADS, smem, st>>>(static_cast<const int4 *>(src), static_cast<int4 *>(dst),
                                                   runs, n_runs, pat16, (uint32_t)units);
    return cudaGetLastError();
}

cudaError_t run_sums(const void *pics, int in_type, size2 src, const uint2 *begins,
                     uint32_t n_rois, size2 slice, uint32_t batch, void *sums, cudaStream_t st,
                     const void *const *ptrs)
{
    const uint32_t n = n_rois * batch;
    if (n == 0) return cudaSuccess;
    if (in_type == IN_U16)
        k_sums<uint16_t><<<n, BLOCK, 0, st>>>(reinterpret_cast<const uint16_t *>(pics), src, begins,
                                              n_rois, slice, reinterpret_cast<uint32_t *>(sums), ptrs);
    else
        k_sums<double><<<n, BLOCK, 0, st>>>(reinterpret_cast<const double *>(pics), src, begins,
                                            n_rois, slice, reinterpret_cast<double *>(sums), ptrs);
    return cudaGetLastError();
}

cudaError_t run_prepare(const void *pics, int in_type, bool dbl, void *out, const void *hann,
                        const void *sums, const uint2 *begins, size2 src, size2 slice,
                        size2 out_size, uint32_t n_rois, uint32_t batch, cudaStream_t st,
                        const void *const *ptrs)
{
    const uint32_t n = n_rois * batch;
    const uint32_t grid = grid_for((uint64_t)n * slice.x * slice.y);
    if (grid == 0) return cudaSuccess;
#define EMIDA_PREP(IN, T)                                                                       \
    k_prepare<IN, T><<<grid, BLOCK, 0, st>>>(                                                   \
        reinterpret_cast<const IN *>(pics), reinterpret_cast<T *>(out),                         \
        reinterpret_cast<const T *>(hann), reinterpret_cast<const sum_of<IN>::type *>(sums),    \
        begins, src, slice, out_size, n_rois, n, ptrs)
    if (in_type == IN_U16) {
        if (dbl) EMIDA_PREP(uint16_t, double);
        else EMIDA_PREP(uint16_t, float);
    } else {
        if (dbl) EMIDA_PREP(double, double);
        else EMIDA_PREP(double, float);
    }
#undef EMIDA_PREP
    return cudaGetLastError();
}

cudaError_t run_cross_corr(const void *pics, const void *ref, void *res, bool dbl, size2 size,
                           size2 res_size, uint32_t ref_slices, uint32_t batch, cudaStream_t st)
{
    const uint32_t n = ref_slices * batch;
    if (n == 0) return cudaSuccess;
    const size_t smem = (size_t)2 * size.x * size.y * (dbl ? 8 : 4);
    if (dbl) {
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(k_cross_corr<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    } else if (smem > 48 * 1024) {
        cudaFuncSetAttribute(k_cross_corr<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    }
    for (uint32_t pair0 = 0; pair0 < n; pair0 += CROSS_CORR_MAX_Y) {
        const dim3 grid(res_size.y, n - pair0 < CROSS_CORR_MAX_Y ? n - pair0 : CROSS_CORR_MAX_Y);
        if (dbl)
            k_cross_corr<double><<<grid, BLOCK, smem, st>>>(
                reinterpret_cast<const double *>(pics), reinterpret_cast<const double *>(ref),
                reinterpret_cast<double *>(res), size, res_size, ref_slices, pair0);
        else
            k_cross_corr<float><<<grid, BLOCK, smem, st>>>(
                reinterpret_cast<const float *>(pics), reinterpret_cast<const float *>(ref),
                reinterpret_cast<float *>(res), size, res_size, ref_slices, pair0);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t run_fft_r2c(const void *real_in, void *spec, uint32_t maps, const fft_tables &t,
                        bool dbl, cudaStream_t st)
{
    const uint32_t half = t.w2 / 2 + 1;
    const uint32_t rows = maps * t.h2, cols = maps * half;
    cudaError_t e;
    if (dbl) {
        e = launch_lines<double>(real_in, spec, LM_R2C_ROWS, -1, (int)t.w2, rows, t.h2, half,
                                 t.w2 * t.h2, half * t.h2, t.tw_row, st);
        if (e == cudaSuccess)
            e = launch_lines<double>(spec, spec, LM_C2C_COLS, -1, (int)t.h2, cols, half, half,
                                     half * t.h2, half * t.h2, t.tw_col, st);
    } else {
        e = launch_lines<float>(real_in, spec, LM_R2C_ROWS, -1, (int)t.w2, rows, t.h2, half,
                                t.w2 * t.h2, half * t.h2, t.tw_row, st);
        if (e == cudaSuccess)
            e = launch_lines<float>(spec, spec, LM_C2C_COLS, -1, (int)t.h2, cols, half, half,
                                    half * t.h2, half * t.h2, t.tw_col, st);
    }
    return e;
}

cudaError_t run_fft_c2r(void *spec, void *real_out, uint32_t maps, const fft_tables &t, bool dbl,
                        cudaStream_t st)
{
    const uint32_t half = t.w2 / 2 + 1;
    const uint32_t rows = maps * t.h2, cols = maps * half;
    cudaError_t e;
    if (dbl) {
        e = launch_lines<double>(spec, spec, LM_C2C_COLS, +1, (int)t.h2, cols, half, half,
                                 half * t.h2, half * t.h2, t.tw_col, st);
        if (e == cudaSuccess)
            e = launch_lines<double>(spec, real_out, LM_C2R_ROWS, +1, (int)t.w2, rows, t.h2, half,
                                     half * t.h2, t.w2 * t.h2, t.tw_row, st);
    } else {
        e = launch_lines<float>(spec, spec, LM_C2C_COLS, +1, (int)t.h2, cols, half, half,
                                half * t.h2, half * t.h2, t.tw_col, st);
        if (e == cudaSuccess)
            e = launch_lines<float>(spec, real_out, LM_C2R_ROWS, +1, (int)t.w2, rows, t.h2, half,
                                    half * t.h2, t.w2 * t.h2, t.tw_row, st);
    }
    return e;
}

cudaError_t run_hadamard(void *pics, const void *ref, uint32_t one_area, uint32_t ref_slices,
                         uint32_t batch, bool dbl, cudaStream_t st)
{
    const uint64_t ref_elems = (uint64_t)one_area * ref_slices, total = ref_elems * batch;
    if (total == 0) return cudaSuccess;
    if (dbl)
        k_hadamard<double><<<grid_for(total), BLOCK, 0, st>>>(
            reinterpret_cast<double2 *>(pics), reinterpret_cast<const double2 *>(ref), ref_elems, total);
    else
        k_hadamard<float><<<grid_for(total), BLOCK, 0, st>>>(
            reinterpret_cast<float2 *>(pics), reinterpret_cast<const float2 *>(ref), ref_elems, total);
    return cudaGetLastError();
}

cudaError_t run_maxarg(const void *maps, uint32_t map_size, uint32_t n, void *maxes, bool dbl,
                       cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    if (dbl)
        k_maxarg<double><<<n, BLOCK, 0, st>>>(reinterpret_cast<const double *>(maps), map_size,
                                              reinterpret_cast<data_index<double> *>(maxes));
    else
        k_maxarg<float><<<n, BLOCK, 0, st>>>(reinterpret_cast<const float *>(maps), map_size,
                                             reinterpret_cast<data_index<float> *>(maxes));
    return cudaGetLastError();
}

cudaError_t run_extract_neighbors(const void *maps, const void *maxes, void *neigh, int s,
                                  size2 cross, uint32_t n, int policy, bool dbl, cudaStream_t st)
{
    const uint64_t total = (uint64_t)n * s * s;
    if (total == 0) return cudaSuccess;
    if (dbl)
        k_extract<double><<<grid_for(total), BLOCK, 0, st>>>(
            reinterpret_cast<const double *>(maps), reinterpret_cast<const data_index<double> *>(maxes),
            reinterpret_cast<double *>(neigh), s, cross, n, policy);
    else
        k_extract<float><<<grid_for(total), BLOCK, 0, st>>>(
            reinterpret_cast<const float *>(maps), reinterpret_cast<const data_index<float> *>(maxes),
            reinterpret_cast<float *>(neigh), s, cross, n, policy);
    return cudaGetLastError();
}

cudaError_t run_fit(const void *neigh, const void *maxes, uint32_t n, int s, size2 cross,
                    int policy, const double *lstsq, bool dbl, double *offsets, double *coefs,
                    cudaStream_t st, const uint32_t *out_base, uint32_t n_rois, void *maxes_out)
{
    if (n == 0) return cudaSuccess;
    if (dbl)
        k_fit<double><<<grid_for(n), BLOCK, 0, st>>>(
            reinterpret_cast<const double *>(neigh), reinterpret_cast<const data_index<double> *>(maxes),
            n, s, cross, policy, lstsq, offsets, coefs, out_base, n_rois,
            reinterpret_cast<data_index<double> *>(maxes_out));
    else
        k_fit<float><<<grid_for(n), BLOCK, 0, st>>>(
            reinterpret_cast<const float *>(neigh), reinterpret_cast<const data_index<float> *>(maxes),
            n, s, cross, policy, lstsq, offsets, coefs, out_base, n_rois,
            reinterpret_cast<data_index<float> *>(maxes_out));
    return cudaGetLastError();
}

cudaError_t run_ref_row_sums(const void *prep, void *spec_cm, uint32_t maps, uint32_t n, bool dbl,
                             cudaStream_t st)
{
    const uint64_t rows = (uint64_t)maps * n, per = (uint64_t)(n / 2 + 1) * n;
    if (rows == 0) return cudaSuccess;
    if (dbl)
        k_ref_row_sums<double><<<grid_for(rows * 32), BLOCK, 0, st>>>(
            reinterpret_cast<const double *>(prep), reinterpret_cast<double2 *>(spec_cm), n, per, rows);
    else
        k_ref_row_sums<float><<<grid_for(rows * 32), BLOCK, 0, st>>>(
            reinterpret_cast<const float *>(prep), reinterpret_cast<float2 *>(spec_cm), n, per, rows);
    return cudaGetLastError();
}

cudaError_t run_spec_to_colmajor(const void *spec, void *out, uint32_t maps, uint32_t w2,
                                 uint32_t h2, bool dbl, cudaStream_t st)
{
    const uint32_t half = w2 / 2 + 1;
    const uint64_t total = (uint64_t)maps * half * h2;
    if (total == 0) return cudaSuccess;
    if (dbl)
        k_to_colmajor<double><<<grid_for(total), BLOCK, 0, st>>>(
            reinterpret_cast<const double2 *>(spec), reinterpret_cast<double2 *>(out), half, h2, total);
    else
        k_to_colmajor<float><<<grid_for(total), BLOCK, 0, st>>>(
            reinterpret_cast<const float2 *>(spec), reinterpret_cast<float2 *>(out), half, h2, total);
    return cudaGetLastError();
}

}  // namespace emida_gb
