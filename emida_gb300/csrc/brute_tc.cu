// brute_tc.cu -- brute-force ROI cross-correlation on the tcgen05 tensor cores.
//
// The reference correlates a 64x64 pattern ROI P with a 64x64 reference ROI R
// over all 127x127 lags by direct summation (src/cross_corr.cu:11-74):
//     res[dy][dx] = sum_{a,x} P[a][x + dx - 63] * R[a - dy + 63][x]
// (out-of-range pixels are zero).  That is one dense GEMM per pair,
//     D[dx][dy] = sum_k A[dx][k] * B[dy][k],  k = (a, x),  M = N = 128, K = 4096,
// with A[dx][(a,x)] = P[a][x + dx - 63] (a Toeplitz matrix per pattern row a)
// and B[dy][(a,x)] = R[a - dy + 63][x].  Both operands are stored in the
// tensor core's no-swizzle K-major form: 8 rows x 16 bytes per core matrix.
//
//   * A: core matrix (dx block i, x block k) of row a holds
//     P[a][8(i + k) + r + c - 63] (row r, column c), so it depends on i + k
//     only.  The 24 distinct core matrices of a row are stored back to back
//     and the descriptor walks both M and K in steps of 128 bytes; a pattern
//     row costs 3 KiB instead of a 128 x 64 materialised Toeplitz block.
//   * B: the reference ROI is stored once per ROI with its rows reversed and
//     64 zero rows either side; the operand of pattern row a is the same
//     buffer at a start offset of -a rows.
//   * Pattern row a meets the reference only at lags dy in [a, a + 63]; the
//     other 64 columns of its B operand are zero rows.  Row 0 runs the full
//     N = 128 (its first product initialises every accumulator column); rows
//     a >= 1 run N = 80 MMAs on the columns [a & ~15, (a & ~15) + 80), which
//     hold that window, at 0.63 of the full tile's products.
//
// Products are BF16 with FP32 accumulation.  Every value is split as
// v = hi + lo (hi = bf16(v), lo = bf16(v - hi)) and D accumulates
// hi*hi + hi*lo + lo*hi, which keeps about 16 significant bits per product.
// Per-ROI sums, means and the Hann window run in FP64 before the split; the
// quadratic fit runs in FP64 (src/subpixel_max.hpp:76-97).
//
// One persistent CTA per SM walks a contiguous range of (ROI, pattern) pairs,
// ROI-major so that the reference operand changes rarely.  Warp roles:
//   warps 0-3  epilogue: TMEM -> registers, argmax (first maximum, as
//              src/maxarg.cu), neighbours (src/extract_neighbors.cu:12-41),
//              fit and the offset (src/gpu_offset.hpp:289-298);
//   warps 4-7  producers: load and prepare the pattern ROI, split it, write
//              the A core matrices of 4 pattern rows per pipeline stage;
//   warp 8     allocates TMEM; lane 0 issues the MMAs.
// The accumulator is double-buffered in TMEM (2 x 128 columns) so the
// epilogue of one pair overlaps the MMAs of the next.  Every wait is bounded:
// when one runs out the kernel records DEV_ERR_WAIT_TIMEOUT, drains its MMAs,
// frees TMEM and returns.
#include <cuda_bf16.h>

#include "brute_tc.cuh"
#include "device_fit.cuh"
#include "ptx.cuh"

namespace emida_gb {
namespace {

using namespace ptx;

constexpr int SIDE = (int)BRUTE_TC_SIDE;
constexpr int CROSS = (int)BRUTE_TC_CROSS;
constexpr int TM = 128, TN = 128;       // MMA tile: dx rows x dy columns
constexpr int WIN_LO = 56, WIN_N = 71;  // 16-byte windows of a pattern row that can hold data
constexpr int A_ROW = 192 * 16;         // 24 core matrices of one pattern row (hi or lo)
constexpr int B_KBLK = 192 * 16;        // one 8-column block of the reference, rows -64..127
constexpr int B_HALF = 8 * B_KBLK;      // hi or lo
constexpr int RPS = 4;                  // pattern rows per pipeline stage
constexpr int NST = 4;                  // stages
constexpr int STAGE = RPS * 2 * A_ROW;
constexpr int PROW = 80;                // prepared pattern row: 8 zeros, 64 values, 8 zeros
constexpr int PROD = 128, EPI = 128;
constexpr int THREADS = EPI + PROD + 32;
constexpr uint32_t TMEM_COLS = 2 * TN;
constexpr uint32_t BAR_PROD = 1, BAR_EPI = 2;  // named barriers

struct smem_layout {
    static constexpr int b_hi = 0;
    static constexpr int b_lo = b_hi + B_HALF;
    static constexpr int a_ring = b_lo + B_HALF;
    static constexpr int p_hi = a_ring + NST * STAGE;
    static constexpr int p_lo = p_hi + SIDE * PROW * 2;
    static constexpr int zero_end = p_lo + SIDE * PROW * 2;  // [0, zero_end) starts at zero
    static constexpr int hann = zero_end;                    // 128 doubles
    static constexpr int neigh = hann + 128 * 8;             // up to 81 floats
    static constexpr int red_val = neigh + 96 * 4;
    static constexpr int red_idx = red_val + 16;
    static constexpr int red_sum = red_idx + 16;
    static constexpr int bars = red_sum + 16;
    static constexpr int n_bars = 2 * NST + 4 + 1;
    static constexpr int tmem_slot = bars + n_bars * 8;
    static constexpr int bytes = tmem_slot + 16;
    static_assert(bars % 8 == 0, "mbarriers are 8-byte aligned");
    static_assert(zero_end % 16 == 0, "zeroed with 16-byte stores");
};
using L = smem_layout;

struct barriers {
    uint64_t *full, *empty, *acc_full, *acc_empty, *drain;
};

__device__ __forceinline__ barriers get_barriers(unsigned char *smem)
{
    uint64_t *b = reinterpret_cast<uint64_t *>(smem + L::bars);
    return barriers{b, b + NST, b + 2 * NST, b + 2 * NST + 2, b + 2 * NST + 4};
}

__device__ __forceinline__ void split_bf16(float f, uint16_t &hi, uint16_t &lo)
{
    const __nv_bfloat16 h = __float2bfloat16_rn(f);
    const __nv_bfloat16 l = __float2bfloat16_rn(f - __bfloat162float(h));
    hi = __bfloat16_as_ushort(h);
    lo = __bfloat16_as_ushort(l);
}

// Producers: pattern ROI -> prepared FP64 -> hi/lo rows -> A core matrices.
__device__ void producer(const brute_tc_args &a, unsigned char *smem, const barriers &bar,
                         uint64_t q0, uint64_t q1, int p)
{
    uint16_t *p_hi = reinterpret_cast<uint16_t *>(smem + L::p_hi);
    uint16_t *p_lo = reinterpret_cast<uint16_t *>(smem + L::p_lo);
    uint32_t *red_sum = reinterpret_cast<uint32_t *>(smem + L::red_sum);
    const double *hann = reinterpret_cast<const double *>(smem + L::hann);
    const int col = p & 63, r0 = p >> 6;
    uint32_t g = 0, k = 0, prev_roi = 0xffffffffu;
    for (uint64_t q = q0; q < q1; ++q, ++k) {
        const uint32_t roi = (uint32_t)(q / a.n_patterns), pat = (uint32_t)(q % a.n_patterns);
        const uint2 bg = a.begins[roi];
        const uint16_t *src = a.pics + (size_t)pat * a.src_w * a.src_h + (size_t)bg.y * a.src_w +
                              bg.x + col;
        uint16_t px[SIDE / 2];
        uint32_t sum = 0;
#pragma unroll
        for (int i = 0; i < SIDE / 2; ++i) {
            px[i] = __ldg(src + (size_t)(r0 + 2 * i) * a.src_w);
            sum += px[i];
        }
        if (roi != prev_roi) {
            // the reference operand is rewritten once the previous pair's MMAs are done
            if (k > 0) {
                bool ok = true;
                if (p == 0) ok = mbar_wait(&bar.acc_full[(k - 1) & 1], ((k - 1) >> 1) & 1);
                if (bar_any(BAR_PROD, PROD, !ok)) {
                    if (p == 0) atomicOr(a.err, (uint32_t)DEV_ERR_WAIT_TIMEOUT);
                    return;
                }
            }
            const double *R = a.ref_prep + (size_t)roi * SIDE * SIDE;
            for (int e = p; e < SIDE * 8; e += PROD) {
                const int kk = e >> 6, b = e & 63;
                uint16_t h[8], l[8];
#pragma unroll
                for (int c = 0; c < 8; ++c) split_bf16((float)R[b * SIDE + kk * 8 + c], h[c], l[c]);
                const int off = kk * B_KBLK + (127 - b) * 16;  // row b' = 63 - b, 64 rows of padding
                *reinterpret_cast<uint4 *>(smem + L::b_hi + off) =
                    make_uint4(h[0] | (h[1] << 16), h[2] | (h[3] << 16), h[4] | (h[5] << 16), h[6] | (h[7] << 16));
                *reinterpret_cast<uint4 *>(smem + L::b_lo + off) =
                    make_uint4(l[0] | (l[1] << 16), l[2] | (l[3] << 16), l[4] | (l[5] << 16), l[6] | (l[7] << 16));
            }
            prev_roi = roi;
        }
        // ROI sum (exact, src/sum.cu) and mean in FP64
#pragma unroll
        for (int off = 16; off; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
        if ((p & 31) == 0) red_sum[p >> 5] = sum;
        bar_sync(BAR_PROD, PROD);
        const uint32_t total = red_sum[0] + red_sum[1] + red_sum[2] + red_sum[3];
        const double mean = (double)total / (double)(SIDE * SIDE);
#pragma unroll
        for (int i = 0; i < SIDE / 2; ++i) {
            const int r = r0 + 2 * i;
            const double v = ((double)px[i] - mean) * hann[col] * hann[SIDE + r];
            uint16_t h, l;
            split_bf16((float)v, h, l);
            p_hi[r * PROW + 8 + col] = h;
            p_lo[r * PROW + 8 + col] = l;
        }
        bar_sync(BAR_PROD, PROD);  // prepared rows (and the reference operand) complete
        for (int st = 0; st < SIDE / RPS; ++st, ++g) {
            const int s = (int)(g % NST);
            bool ok = true;
            if (p == 0) ok = mbar_wait(&bar.empty[s], ((g / NST) & 1) ^ 1);
            if (bar_any(BAR_PROD, PROD, !ok)) {
                if (p == 0) atomicOr(a.err, (uint32_t)DEV_ERR_WAIT_TIMEOUT);
                return;
            }
            unsigned char *stage = smem + L::a_ring + s * STAGE;
            for (int e = p; e < RPS * 2 * WIN_N; e += PROD) {
                const int rr = e / (2 * WIN_N), rem = e % (2 * WIN_N);
                const int lo = rem >= WIN_N;
                const int w = WIN_LO + (lo ? rem - WIN_N : rem);
                // window w of row a holds P[a][w - 63 .. w - 56] = prepared row slots w-55 .. w-48
                const uint16_t *s8 = (lo ? p_lo : p_hi) + (st * RPS + rr) * PROW + (w - 55);
                *reinterpret_cast<uint4 *>(stage + rr * 2 * A_ROW + lo * A_ROW + w * 16) =
                    make_uint4(s8[0] | ((uint32_t)s8[1] << 16), s8[2] | ((uint32_t)s8[3] << 16),
                               s8[4] | ((uint32_t)s8[5] << 16), s8[6] | ((uint32_t)s8[7] << 16));
            }
            fence_proxy_async();
            mbar_arrive(&bar.full[s]);
        }
    }
}

// Lane 0 of warp 8: 64 pattern rows x 4 K-steps x 3 split products per pair,
// on the accumulator columns that pattern row can reach.
constexpr int TN_WIN = 80;  // lag columns of a pattern row's window: 64 + 15, rounded to 16
__device__ void mma_issuer(const brute_tc_args &a, unsigned char *smem, const barriers &bar,
                           uint64_t q0, uint64_t q1, uint32_t tmem)
{
    constexpr uint32_t idesc = idesc_bf16_f32(TM, TN);
    constexpr uint32_t idesc_win = idesc_bf16_f32(TM, TN_WIN);
    // Every operand address is a base plus a constant, and a descriptor's low
    // 14 bits are the address / 16, so each descriptor below is a base
    // descriptor plus a small integer: the single issuing thread spends a few
    // adds per MMA instead of rebuilding four 64-bit descriptors.
    const uint64_t dA0 = smem_desc(smem_u32(smem + L::a_ring), 128, 128);
    const uint64_t dBh0 = smem_desc(smem_u32(smem + L::b_hi) + 64 * 16, B_KBLK, 128);  // pattern row 0
    const uint64_t dBl0 = smem_desc(smem_u32(smem + L::b_lo) + 64 * 16, B_KBLK, 128);
    uint32_t g = 0, k = 0;
    bool ok = true;
    for (uint64_t q = q0; q < q1 && ok; ++q, ++k) {
        const uint32_t b = k & 1;
        if (!(ok = mbar_wait(&bar.acc_empty[b], ((k >> 1) & 1) ^ 1))) break;
        tc_fence_after();
        const uint32_t d = tmem + b * TN;
        for (int st = 0; st < SIDE / RPS; ++st, ++g) {
            const int s = (int)(g % NST);
            if (!(ok = mbar_wait(&bar.full[s], (g / NST) & 1))) break;
            tc_fence_after();
            const uint64_t dAs = dA0 + (uint64_t)((s * STAGE) >> 4);
#pragma unroll
            for (int rr = 0; rr < RPS; ++rr) {
                const int row = st * RPS + rr;  // B starts row rows earlier
                // row 0: all 128 lag columns; later rows: the 80 from row & ~15
                const uint32_t dy0 = row == 0 ? 0u : (uint32_t)(row & ~15);
                const uint32_t id = row == 0 ? idesc : idesc_win;
#pragma unroll
                for (int ks = 0; ks < SIDE / 16; ++ks) {
                    const uint64_t dah = dAs + ((rr * 2 * A_ROW + ks * 256) >> 4);
                    const uint64_t dal = dah + (A_ROW >> 4);
                    const uint64_t dbh = dBh0 - (uint64_t)row + dy0 + ((ks * 2 * B_KBLK) >> 4);
                    const uint64_t dbl = dBl0 - (uint64_t)row + dy0 + ((ks * 2 * B_KBLK) >> 4);
                    mma_bf16(d + dy0, dah, dbh, id, (row | ks) != 0);
                    mma_bf16(d + dy0, dah, dbl, id, 1);
                    mma_bf16(d + dy0, dal, dbh, id, 1);
                }
            }
            mma_commit(&bar.empty[s]);
        }
        if (ok) mma_commit(&bar.acc_full[b]);
    }
    if (!ok) atomicOr(a.err, (uint32_t)DEV_ERR_WAIT_TIMEOUT);
    // everything issued must be complete before TMEM is released
    mma_commit(bar.drain);
    if (!mbar_wait(bar.drain, 0)) atomicOr(a.err, (uint32_t)DEV_ERR_WAIT_TIMEOUT);
}

__device__ void epilogue(const brute_tc_args &a, unsigned char *smem, const barriers &bar,
                         uint64_t q0, uint64_t q1, uint32_t tmem, int e)
{
    const int warp = e >> 5, lane = e & 31;
    float *neigh = reinterpret_cast<float *>(smem + L::neigh);
    float *red_val = reinterpret_cast<float *>(smem + L::red_val);
    uint32_t *red_idx = reinterpret_cast<uint32_t *>(smem + L::red_idx);
    const int s = a.fitsize, s2 = s * s;
    uint32_t k = 0;
    for (uint64_t q = q0; q < q1; ++q, ++k) {
        const uint32_t roi = (uint32_t)(q / a.n_patterns), pat = (uint32_t)(q % a.n_patterns);
        const uint32_t b = k & 1;
        bool ok = true;
        if (e == 0) ok = mbar_wait(&bar.acc_full[b], (k >> 1) & 1);
        if (bar_any(BAR_EPI, EPI, !ok)) {
            if (e == 0) atomicOr(a.err, (uint32_t)DEV_ERR_WAIT_TIMEOUT);
            return;
        }
        tc_fence_after();
        // lane e of the accumulator is lag column dx = e; TMEM column dy is the lag row
        const uint32_t tbase = tmem + ((uint32_t)(warp * 32) << 16) + b * TN;
        float best = -__int_as_float(0x7f800000);
        uint32_t bi = 0xffffffffu;
#pragma unroll
        for (int c = 0; c < TN / 32; ++c) {
            float v[32];
            tmem_ld32(tbase + c * 32, v);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int dy = c * 32 + j;
                if (dy < CROSS && e < CROSS && v[j] > best) {
                    best = v[j];
                    bi = (uint32_t)(dy * CROSS + e);
                }
            }
        }
#pragma unroll
        for (int off = 16; off; off >>= 1) {
            const float ov = __shfl_xor_sync(0xffffffffu, best, off);
            const uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ov > best || (ov == best && oi < bi)) {
                best = ov;
                bi = oi;
            }
        }
        if (lane == 0) {
            red_val[warp] = best;
            red_idx[warp] = bi;
        }
        bar_sync(BAR_EPI, EPI);
        float bv = red_val[0];
        uint32_t bidx = red_idx[0];
        for (int w = 1; w < 4; ++w)
            if (red_val[w] > bv || (red_val[w] == bv && red_idx[w] < bidx)) {
                bv = red_val[w];
                bidx = red_idx[w];
            }
        const uint32_t mx = bidx % CROSS, my = bidx / CROSS;
        // s x s neighbours, clamped to [0, cross] as the reference does; a
        // clamped position is read at its linear index in the 127 x 127 map
        for (int t = 0; t < s2; ++t) {
            uint32_t x, y;
            neighbour_pos(mx, my, t % s, t / s, s, CROSS, CROSS, x, y);
            const uint32_t lin = y * CROSS + x;
            if (lin < (uint32_t)(CROSS * CROSS)) {
                const uint32_t xx = lin % CROSS, yy = lin / CROSS;
                const float v = tmem_ld1(tbase + yy);
                if ((uint32_t)e == xx) neigh[t] = v;
            } else if (e == 0) {
                neigh[t] = 0.f;  // past the end of this map
            }
        }
        tc_fence_before();
        mbar_arrive(&bar.acc_empty[b]);
        bar_sync(BAR_EPI, EPI);
        if (warp == 0) {
            const size_t slot = (size_t)pat * a.n_rois + roi;
            double c = 0.0;
            if (lane < 6) {
                const double *m = a.lstsq + lane * s2;
                for (int t = 0; t < s2; ++t) c = __dadd_rn(c, __dmul_rn(m[t], (double)neigh[t]));
            }
            double cs[6];
#pragma unroll
            for (int j = 0; j < 6; ++j) cs[j] = __shfl_sync(0xffffffffu, c, j);
            if (lane == 0) {
                double ox, oy;
                fit_offsets(cs, mx, my, CROSS, CROSS, s, ox, oy);
                a.offsets[2 * slot] = ox;
                a.offsets[2 * slot + 1] = oy;
                if (a.coefs)
                    for (int j = 0; j < 6; ++j) a.coefs[6 * slot + j] = cs[j];
                if (a.maxes) {
                    data_index<float> *mi = reinterpret_cast<data_index<float> *>(a.maxes) + slot;
                    mi->data = bv;
                    mi->index = bidx;
                }
            }
            if (a.neigh)
                for (int t = lane; t < s2; t += 32) a.neigh[slot * s2 + t] = neigh[t];
        }
    }
}

__global__ void __launch_bounds__(THREADS, 1) brute_tc_kernel(const brute_tc_args a)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const int warp = threadIdx.x >> 5;
    const barriers bar = get_barriers(smem);
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(smem + L::tmem_slot);
    double *hann = reinterpret_cast<double *>(smem + L::hann);

    for (int i = threadIdx.x; i < L::zero_end / 16; i += THREADS)
        reinterpret_cast<uint4 *>(smem)[i] = make_uint4(0, 0, 0, 0);
    for (int i = threadIdx.x; i < 2 * SIDE; i += THREADS) hann[i] = a.hann[i];
    if (threadIdx.x == 0) {
        for (int s = 0; s < NST; ++s) {
            mbar_init(&bar.full[s], PROD);
            mbar_init(&bar.empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&bar.acc_full[b], 1);
            mbar_init(&bar.acc_empty[b], EPI);
        }
        mbar_init(bar.drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_proxy_async();  // the zeroed operand padding is read by the tensor core
    if (warp == 8) tmem_alloc(tmem_slot, TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    const uint64_t total = (uint64_t)a.n_patterns * a.n_rois;
    const uint64_t q0 = total * blockIdx.x / gridDim.x;
    const uint64_t q1 = total * (blockIdx.x + 1) / gridDim.x;
    if (warp >= 4 && warp < 8)
        producer(a, smem, bar, q0, q1, (int)threadIdx.x - EPI);
    else if (warp == 8) {
        if ((threadIdx.x & 31) == 0) mma_issuer(a, smem, bar, q0, q1, tmem);
        __syncwarp();
    } else
        epilogue(a, smem, bar, q0, q1, tmem, (int)threadIdx.x);

    tc_fence_before();
    __syncthreads();
    if (warp == 8) {
        tc_fence_after();
        tmem_dealloc(tmem, TMEM_COLS);
    }
}

}  // namespace

cudaError_t launch_brute_tc(const brute_tc_args &a, int grid, cudaStream_t st)
{
    const uint64_t total = (uint64_t)a.n_patterns * a.n_rois;
    if (total == 0) return cudaSuccess;
    if (a.fitsize != 3 && a.fitsize != 5 && a.fitsize != 7 && a.fitsize != 9)
        return cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(brute_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, L::bytes);
    if (e != cudaSuccess) return e;
    if (grid <= 0) grid = sms + grid > 1 ? sms + grid : 1;
    if ((uint64_t)grid > total) grid = (int)total;
    brute_tc_kernel<<<grid, THREADS, L::bytes, st>>>(a);
    return cudaGetLastError();
}

size_t brute_tc_smem_bytes() { return L::bytes; }

cudaError_t preload_brute_tc()
{
    return cudaFuncSetAttribute(brute_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, L::bytes);
}

}  // namespace emida_gb
