// fused.cu -- the fused FFT-policy kernel: one CTA carries one (pattern, ROI)
// pair at a time through the whole path of src/gpu_offset.hpp:234-301 --
//   ROI gather (TMA) -> sum -> mean/Hann (prepare_pics.cu:34-41)
//   -> 2N x 2N R2C in shared memory -> conj product with the resident reference
//   spectrum (hadamard.cu:39-40) -> C2R -> argmax (maxarg.cu, first maximum)
//   -> s x s neighbourhood (extract_neighbors.cu, FFT index policy)
//   -> FP64 fit and offset (subpixel_max.hpp:76-97, gpu_offset.hpp:289-298).
// Nothing but the ROI pixels is read from HBM per pair and nothing but the
// results is written back; the reference spectra (66.5 KB per ROI at N=128)
// stay L2-resident across the batch.
//
// Shared-memory spectrum: N rows (ky) x N/2 complex slots (kx), slot 0 packs
// the real DC and Nyquist columns as (X[.][0], X[.][N/2]).  Slots are XOR
// swizzled by row so that column and row accesses of the 8-lane FFT groups
// spread over all banks.  The uint16 ROI tile is staged by TMA into the
// spectrum's upper half, which is unused until the column pass.
#include <cooperative_groups.h>
#include <cstring>
#include <cuda.h>

#include "device_fit.cuh"
#include "fft.cuh"
#include "fused.cuh"

namespace emida_gb {

namespace {

// Slot swizzle: XOR the slot with f(row & 7), f = 2 * (row bits 0, 2, 1 as bits
// 0, 1, 2).  64-bit accesses are served per half-warp (two 8-lane groups).
// A group's column access (8 rows t + 8m of one column) gets 8 distinct even
// slot offsets, and its neighbour group's column (c + 1) the odd ones.  Two
// groups' row accesses (rows 8w + 2g' + e) land in different 8-slot halves.
// So every half-warp access covers 16 distinct 8-byte slots.
//
// The 96-point kernel's FFT groups are 4 lanes wide, so a half-warp holds four
// groups: its column accesses cover 4 rows of 4 adjacent columns, its row
// accesses the same slots of rows 2g and 2g + 1 of four groups g.  There
// f = 4 ((row ^ row >> 1) mod 4) gives each of those 4 rows its own 4-slot
// block.  Both forms change slot bits 1-3 only, so a slot stays in its row.
//
// FP64 slots are 16 bytes, so an access is served per quarter-warp, one 8-lane
// group, over 8 bank groups: f = row mod 8 gives a group's column access (8
// rows of one column) 8 distinct slots mod 8, and leaves its row accesses
// (consecutive slots) distinct.
template <int N, typename C>
__device__ __forceinline__ C *sp(C *S, int row, int slot)
{
    const int f = N == 96 ? ((row ^ (row >> 1)) & 3) << 2
                  : sizeof(C) == 16 ? (row & 7)
                                    : ((row & 1) << 1) | (row & 4) | ((row & 2) << 2);
    return S + row * (N / 2) + (slot ^ f);
}

// The correlation map replaces the spectrum: map rows 2p and 2p + 1 at column x
// are one complex slot, (map[2p][x], map[2p + 1][x]), in spectrum rows 2p
// (x < N/2) and 2p + 1 (x >= N/2): one 8- or 16-byte store per lane and
// column instead of two.
template <int N, typename C> __device__ __forceinline__ C *map_pair(C *S, int row2, int x)
{
    return x >= N / 2 ? sp<N>(S, row2 + 1, x - N / 2) : sp<N>(S, row2, x);
}

// Rows 2p and 2p+1 differ in one swizzle bit (every length but 96), so for the
// slots t + 8j a lane touches in both rows, the second row's address is the
// first's plus a per-lane constant: (slot ^ f(2p) ^ d) - (slot ^ f(2p)) is +-d
// by bit d of slot ^ f(2p), and that bit does not depend on j.
template <int N, typename C> __device__ __forceinline__ ptrdiff_t pair_row_delta(C *S, int row2, int slot)
{
    return sp<N>(S, row2 + 1, slot) - sp<N>(S, row2, slot);
}

template <int N, typename C> struct col_line {
    C *S;
    int c;
    __device__ __forceinline__ C *operator()(int q) const { return sp<N>(S, q, c); }
};
template <int N, typename C> struct row_line {
    C *S;
    int a;
    __device__ __forceinline__ C *operator()(int q) const
    {
        return q >= N / 2 ? sp<N>(S, a + 1, q - N / 2) : sp<N>(S, a, q);
    }
};

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
// 16 bytes global -> shared, cached in L2 only; completion is tracked by
// cp_async_arrive on an mbarrier.
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// The mbarrier counts one arrival of this thread once all its earlier
// cp.async copies have landed (the barrier's expected count includes it).
__device__ __forceinline__ void cp_async_arrive(uint64_t *bar)
{
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Bounded wait on an mbarrier phase: returns false when the budget ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    const long long budget = 4000000000LL; /* ~2 s at 2 GHz */
    long long start = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;"
            " selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - start > budget) return false;
    }
}

template <typename T> __device__ __forceinline__ T neg_inf();
template <> __device__ __forceinline__ float neg_inf<float>() { return -__int_as_float(0x7f800000); }
template <> __device__ __forceinline__ double neg_inf<double>()
{
    return -__longlong_as_double(0x7ff0000000000000LL);
}

template <typename T>
__device__ __forceinline__ void better(T &bv, uint32_t &bi, T v, uint32_t i)
{
    if (v > bv || (v == bv && i < bi)) {
        bv = v;
        bi = i;
    }
}

}  // namespace

// The conj product of column c (1 <= c < N/2) of the spectrum (held in v, E
// values per lane of the group) with its reference column, in place.
template <int N, int G, typename T>
__device__ __forceinline__ void conj_product(cplx<T> *v, const cplx<T> *R, int c, int t)
{
    constexpr int E = N / G;
    const cplx<T> *Rc = R + (size_t)c * N;
#pragma unroll
    for (int j = 0; j < E; ++j) v[j] = cmulc(v[j], __ldg(Rc + t + G * j));
}

// Slot 0 of every spectrum row packs the real DC and Nyquist columns (kx = 0
// and N/2).  Their products with the reference and inverse column transforms
// are two real 1-D circular correlations along ky, computed directly: with d,
// q the DC and Nyquist outputs of the row pass (zero for y >= side) and r0, r1
// the reference ROI's row sums and alternating row sums (staged from column 0
// of the resident reference),
//   IFFT(FFT(d) conj(FFT(r0)))[tau] = N sum_{b < side} d[(b + tau) mod N] r0[b],
// the unnormalised inverse of the FFT path; likewise for q and r1.
// Planar layout: dq[c * DQ + y] = component c (d, q) at y mod N for y < DQ, so
// no index wraps; rs[c * N/2 + b] = r_c[b].  The 2N outputs form N/2 blocks of
// 4 consecutive tau of one component; Q = THREADS / (N/2) consecutive lanes
// share a block, each summing a contiguous part of the b range with a sliding
// window of 4 values, and combine by shuffles.  Lane q's part starts at
// b = q (mod Q): the lanes' window heads 4 * block + b then fall in distinct
// banks.  Lane q of the block writes outputs q, q + Q, ... to slot 0.
template <int N> constexpr int packed_dq() { return 3 * N / 2 + 4; }
// NCOMP components from comp_first on; slot0(tau) is the slot-0 entry of row
// tau (in this CTA's spectrum, or in the partner's through distributed shared
// memory).
template <int N, int THREADS, int NCOMP, typename T, typename Slot0>
__device__ __forceinline__ void packed_column(const Slot0 &slot0, const T *dq, const T *rs, int side, int tid,
                                              int comp_first)
{
    constexpr int Q = THREADS / (NCOMP * N / 4), DQ = packed_dq<N>();
    static_assert(Q == 2 || Q == 4, "lanes per block of 4 lags");
    const int q = tid % Q, blk = tid / Q;
    const int comp = comp_first + blk / (N / 4), tau0 = 4 * (blk % (N / 4));
    const T *dv = dq + comp * DQ;
    const T *rv = rs + comp * (N / 2);
    auto start = [&](int k) {
        const int b = (k * side / Q) / Q * Q + k;
        return b < side ? b : side;
    };
    const int b0 = start(q), b1 = q + 1 < Q ? start(q + 1) : side;
    T w0 = dv[tau0 + b0], w1 = dv[tau0 + b0 + 1], w2 = dv[tau0 + b0 + 2];
    T a0 = (T)0, a1 = (T)0, a2 = (T)0, a3 = (T)0;
#pragma unroll 4
    for (int b = b0; b < b1; ++b) {
        const T w3 = dv[tau0 + b + 3];
        const T r = rv[b];
        a0 += w0 * r;
        a1 += w1 * r;
        a2 += w2 * r;
        a3 += w3 * r;
        w0 = w1;
        w1 = w2;
        w2 = w3;
    }
#pragma unroll
    for (int o = 1; o < Q; o <<= 1) {
        a0 += __shfl_xor_sync(0xffffffffu, a0, o);
        a1 += __shfl_xor_sync(0xffffffffu, a1, o);
        a2 += __shfl_xor_sync(0xffffffffu, a2, o);
        a3 += __shfl_xor_sync(0xffffffffu, a3, o);
    }
#pragma unroll
    for (int k = 0; k < 4; k += Q) {
        const int j = k + q;  // this lane's output of the block
        const T v = j == 0 ? a0 : j == 1 ? a1 : j == 2 ? a2 : a3;
        reinterpret_cast<T *>(slot0(tau0 + j))[comp] = v * (T)N;
    }
}

// Resident CTAs per SM the register budget is sized for (shared memory allows
// as many): FP32 128-point and 192-point transforms are register-heavy; the
// FP32 64-point kernel (8 values per lane) fits 80 registers, so 6 CTAs of 4
// warps share an SM (65 M pairs/s at side 32, against 52 M with 4).
__host__ __device__ constexpr int fused_min_blocks(int N, int tsize, int ppc = 1)
{
    return N == 96 && tsize == 4 ? 4 / ppc
           : N == 192 ? 1 : N == 128 ? (tsize == 4 ? 2 : 1) : N == 64 && tsize == 4 ? 6 : (tsize == 4 ? 4 : 2);
}
// Pairs one CTA carries side by side.  The FP32 96-point kernel's 3-warp
// pairs ran 4 CTAs per SM, each in its own pass of the loop, and their
// instruction working set outgrew the instruction cache; 4 pairs per CTA
// keep the SM's warps in the same pass.  Each pair has its own shared-memory
// block, barrier and warps; the CTA's barriers are common.  That kernel is
// also built with 1 and 2 pairs per CTA, for the multi-layout autotuner.
template <int N, typename T> constexpr int fused_pairs_per_cta() { return N == 96 && sizeof(T) == 4 ? 4 : 1; }

// Lane l fits buffered pair l: coefficients as sequential FP64 dot products
// and the closed-form extremum (src/subpixel_max.hpp:14-29, :76-97), offset
// (src/gpu_offset.hpp:296-297).  One warp instruction serves up to 32 pairs,
// which matters on a part whose FP64 pipe is narrow.
template <typename T>
__device__ __forceinline__ void fit_batch(const fused_args &a, const T *fbuf, const uint32_t *fmeta,
                                          const T *fval, int count, int lane, uint32_t cross)
{
    if (lane < count) {
        const uint32_t pair = fmeta[4 * lane], mxy = fmeta[4 * lane + 1], pks = fmeta[4 * lane + 2];
        const uint32_t mx = mxy & 0xffffu, my = mxy >> 16;
        const int s = (int)(pks >> 24), s2 = s * s;
        const double *lstsq = a.items ? a.lstsq_all + lstsq_offset(s) : a.lstsq;
        double v[81];
        for (int k = 0; k < s2; ++k) v[k] = (double)fbuf[lane * 81 + k];
        double c[6];
        for (int j = 0; j < 6; ++j) c[j] = fit_coef(lstsq, v, s, j);
        double ox, oy;
        fit_offsets(c, mx, my, cross, cross, s, ox, oy);
        a.offsets[2 * (size_t)pair] = ox;
        a.offsets[2 * (size_t)pair + 1] = oy;
        if (a.coefs)
            for (int j = 0; j < 6; ++j) a.coefs[(size_t)pair * 6 + j] = c[j];
        if (a.maxes) {
            data_index<T> *mi = reinterpret_cast<data_index<T> *>(a.maxes) + pair;
            mi->data = fval[lane];
            mi->index = pks & 0xffffffu;
        }
    }
    __syncwarp();
}

// Shared-memory layout of the fused kernel, in bytes from the (1024-aligned)
// dynamic base.  The kernel and the launcher's size both come from here.
template <int N, int G, typename T, int PPC_ = fused_pairs_per_cta<N, T>()> struct fused_layout {
    using C = cplx<T>;
    static constexpr size_t up(size_t v, size_t a) { return (v + a - 1) / a * a; }
    static constexpr size_t spectrum = 0;                                  // N x N/2 C
    static constexpr size_t tw_fwd = spectrum + (size_t)N * (N / 2) * sizeof(C);
    static constexpr size_t tw_bytes = (size_t)G * tw_stride<N, G, C>() * sizeof(C);  // [G][TS]
    static constexpr size_t tw_inv = tw_fwd + tw_bytes;
    static constexpr size_t hann = tw_inv + tw_bytes;
    static constexpr size_t dq = hann + (size_t)N * sizeof(T);            // hx, hy
    static constexpr size_t rsum = dq + (size_t)packed_dq<N>() * sizeof(C);  // DC, Nyquist
    static constexpr size_t red_val = rsum + (size_t)(N / 2) * sizeof(C); // reference row sums
    static constexpr size_t red_idx = red_val + 32 * sizeof(T);
    static constexpr size_t red_sum = up(red_idx + 32 * sizeof(uint32_t), 8);
    // the tile's mbarrier, then (first pair's block) the round the pair queue handed out
    static constexpr size_t barrier = red_sum + 32 * sizeof(double);
    static constexpr size_t next_pair = barrier + 8;
    static constexpr size_t fit_vals = barrier + 16;
    static constexpr size_t fit_meta = up(fit_vals + 32 * 81 * sizeof(T), 4);
    static constexpr size_t fit_peak = up(fit_meta + 32 * 4 * sizeof(uint32_t), sizeof(T));
    static constexpr size_t tile = up(fit_peak + 32 * sizeof(T), 128);
    static constexpr size_t pair_end = tile + (size_t)(N / 2) * (N / 2 + 8) * sizeof(uint16_t);
    static constexpr int PPC = PPC_;
    static constexpr size_t pair_bytes = up(pair_end, 128);  // one pair's block
    static constexpr size_t bytes = PPC == 1 ? pair_end : PPC * pair_bytes;
    static_assert(G * (N / G) == N, "group width must divide the transform length");
    // the FP64-input ROI is staged in the spectrum's upper half
    static_assert((size_t)(N / 2) * (N / 2) * sizeof(double) <=
                      (size_t)(N / 2) * (N / 2) * sizeof(C), "FP64 tile must fit");
};

template <int N, int G, typename T, typename IN, int PPC_>
__global__ void __launch_bounds__(N * G / 4 * PPC_, fused_min_blocks(N, sizeof(T), PPC_))
    fused_fft_kernel(const fused_args a, const __grid_constant__ CUtensorMap tmap)
{
    using C = cplx<T>;
    constexpr int H = N / 2;           // ROI side
    constexpr int SL = N / 2;          // slots per spectrum row
    constexpr int E = N / G;           // elements per lane
    constexpr int GROUPS = N / 4;      // one pair of ROI rows per group in the row pass
    constexpr int THREADS = GROUPS * G;
    constexpr int WARPS = THREADS / 32;
    // ROI side (<= H): smaller ROIs are zero-padded into this transform length
    const int side = a.side;
    // uint16 tile row = TMA box width: covers x offsets 0..7 and keeps the box
    // a whole number of 16-byte units
    const int TW = (side + 14) & ~7;
    constexpr bool U16 = sizeof(IN) == 2;

    using L = fused_layout<N, G, T, PPC_>;
    constexpr int PPC = L::PPC;
    extern __shared__ __align__(1024) unsigned char smem[];
    // this thread's pair of the CTA's PPC and that pair's shared-memory block
    const int sub = PPC == 1 ? 0 : (int)threadIdx.x / THREADS;
    unsigned char *base = smem + (size_t)sub * L::pair_bytes;
    C *S = reinterpret_cast<C *>(base + L::spectrum);
    C *twf = reinterpret_cast<C *>(base + L::tw_fwd);   // [G][TS] forward inter-pass twiddles
    C *twi = reinterpret_cast<C *>(base + L::tw_inv);   // [G][TS] inverse
    T *hx = reinterpret_cast<T *>(base + L::hann);      // hx[H] then hy[H]
    T *hy = hx + a.side;
    constexpr int DQ = packed_dq<N>();
    T *dq = reinterpret_cast<T *>(base + L::dq);         // the row pass's DC and Nyquist outputs
    T *rs = reinterpret_cast<T *>(base + L::rsum);       // the reference's row sums (this ROI)
    T *red_v = reinterpret_cast<T *>(base + L::red_val);
    uint32_t *red_i = reinterpret_cast<uint32_t *>(base + L::red_idx);
    double *red_s = reinterpret_cast<double *>(base + L::red_sum);
    uint64_t *bar = reinterpret_cast<uint64_t *>(base + L::barrier);
    // the round the pair queue handed out, in the first pair's block
    uint32_t *next_s = reinterpret_cast<uint32_t *>((PPC == 1 ? base : smem) + L::next_pair);
    // neighbourhoods of up to 32 pairs wait here for one lane-per-pair fit
    T *fbuf = reinterpret_cast<T *>(base + L::fit_vals);            // [32][81]
    uint32_t *fmeta = reinterpret_cast<uint32_t *>(base + L::fit_meta);  // [32][4]
    T *fval = reinterpret_cast<T *>(base + L::fit_peak);            // [32]
    // uint16 ROIs: a tile of their own (128-byte aligned), refilled by TMA for
    // the next pair while this pair is in its column and inverse passes.
    // FP64 ROIs: staged in the spectrum's upper half, unused until the columns.
    uint16_t *t16 = reinterpret_cast<uint16_t *>(base + L::tile);
    double *t64 = reinterpret_cast<double *>(S + H * SL);

    // thread index within the pair (threads of one pair share no warp with another's)
    const int tid = PPC == 1 ? (int)threadIdx.x : (int)threadIdx.x % THREADS;
    const int lane = tid & 31, warp = tid >> 5;
    const int t = lane & (G - 1), g = tid / G;
    static_assert(THREADS % 32 == 0, "whole warps per pair");

    const C *gtw = reinterpret_cast<const C *>(a.twiddles);
    constexpr int TS = tw_stride<N, G, C>();
    for (int i = tid; i < G * TS; i += THREADS) {
        const int k1 = i % TS;  // W_N^{t k1}, t = i / TS (the row's padding is zero)
        const C w = k1 < E ? gtw[(i / TS) * k1] : cmake<C>((T)0, (T)0);
        twf[i] = w;
        twi[i] = cconj(w);
    }
    const T *ghann = reinterpret_cast<const T *>(a.hann);
    for (int i = tid; i < 2 * a.side; i += THREADS) hx[i] = ghann[i];  // hx then hy
    // rows N/2..N-1 of the DC and Nyquist columns are the zero padding, as is
    // the tail past their copy at N..3N/2-1; the row pass writes rows
    // 0..N/2-1 and that copy for every pair
    for (int i = tid; i < 2 * DQ; i += THREADS) {
        const int y = i % DQ;
        if ((y >= N / 2 && y < N) || y >= 3 * N / 2) dq[i] = (T)0;
    }
    const bool tma = U16 && a.stage == STAGE_TMA;
    const bool cpa = U16 && a.stage == STAGE_ASYNC;
    if (tid == 0) {
        // TMA: one arrival (with the byte count) per tile; cp.async: one per thread
        mbar_init(bar, cpa ? THREADS : 1);
        fence_proxy_async();
    }
    __syncthreads();

    // pair -> (pattern, ROI, output slot, fit size)
    auto item = [&](uint32_t pair) -> uint4 {
        if (a.items) return a.items[pair];
        return make_uint4(pair / a.n_rois, pair % a.n_rois, pair, (uint32_t)a.fitsize);
    };
    auto pattern_base = [&](uint32_t pic) -> const IN * {
        if (a.pattern_ptrs) return reinterpret_cast<const IN *>(a.pattern_ptrs[pic]);
        return reinterpret_cast<const IN *>(a.pics) + (size_t)pic * a.src_w * a.src_h;
    };
    auto issue_tile = [&](uint32_t pair) {
        const uint4 it = item(pair);
        const uint32_t pic = it.x;
        const uint2 b = a.begins[it.y];
        fence_proxy_async();
        mbar_expect_tx(bar, TW * side * 2);
        tma_load_3d(t16, &tmap, (int)(b.x & ~7u), (int)b.y, (int)pic, bar);
    };
    // cp.async staging: every thread copies some of the tile's 16-byte chunks,
    // [x & ~7, roundup(x + side, 8)) of each ROI row, to the layout TMA uses
    // (the ROI starts at column x & 7), then arrives on the barrier
    auto issue_chunks = [&](uint32_t pair) {
        const uint4 it = item(pair);
        const uint2 b = a.begins[it.y];
        const uint16_t *src = reinterpret_cast<const uint16_t *>(pattern_base(it.x)) +
                              (size_t)b.y * a.src_w + (b.x & ~7u);
        const int nch = ((int)(b.x & 7u) + side + 7) >> 3;
        for (int i = tid; i < side * nch; i += THREADS) {
            const int r = i / nch, c = i - r * nch;
            cp_async16(t16 + r * TW + 8 * c, src + (size_t)r * a.src_w + 8 * c);
        }
        cp_async_arrive(bar);
    };
    // the CTA's pairs: PPC consecutive ones per round, rounds gridDim.x * PPC
    // apart; with a pair queue, the first round blockIdx.x and then whichever
    // round the queue hands out (the queue counts rounds of PPC pairs)
    const uint32_t stride = gridDim.x * PPC;
    uint32_t *const queue = a.pair_queue;
    const bool lead = sub == 0 && tid == 0;  // the CTA's thread 0: it talks to the queue
    const uint32_t first = blockIdx.x * PPC + sub;
    if (tma && tid == 0 && first < a.n_pairs) issue_tile(first);
    if (cpa && first < a.n_pairs) issue_chunks(first);

    // uint16 tiles staged ahead (TMA or cp.async): warps 1..WARPS-1 sum the next
    // pair's tile while warp 0 finishes the current pair, so the next pair
    // starts from their partial sums without a summing pass and its barrier
    const bool sum_ahead = U16 && (tma || cpa);
    uint32_t *red_u = reinterpret_cast<uint32_t *>(red_s);  // next tile's partial sums
    bool summed = false;  // this pair's tile was summed ahead (uniform over the CTA)
    uint32_t iter = 0;
    // each pair's ROI corner is loaded during the pair before it
    uint2 beg_next = first < a.n_pairs ? a.begins[item(first).y] : make_uint2(0, 0);
    for (uint32_t round0 = blockIdx.x * PPC, nround = 0; round0 < a.n_pairs; round0 = nround, ++iter) {
        // the queue's answer is needed after the row pass, which hides its latency
        uint32_t fetched = 0;
        if (queue && lead) fetched = (atomicAdd(queue, 1u) + gridDim.x) * PPC;
        // only the last round can leave some of the CTA's pairs without one:
        // they run it on a copy of the last pair and write nothing
        const uint32_t mine = round0 + sub;
        const bool live = mine < a.n_pairs;
        const uint32_t pair = live ? mine : a.n_pairs - 1;
        const uint4 it = item(pair);
        const uint32_t pic = it.x, roi = it.y, out = it.z;
        const int s = (int)it.w, s2 = s * s;
        const uint2 beg = beg_next;

        // ---- gather the ROI and sum it (sum.cu:109-158) -------------------
        T mean;
        const int xo = U16 ? (int)(beg.x & 7u) : 0;
        if constexpr (U16) {
            if (tma || cpa) {
                const bool ok = !live || mbar_wait(bar, iter & 1);
                bool stop = !ok;
                // the CTA's pairs leave together, so no barrier waits for a pair gone
                if constexpr (PPC > 1) stop = __syncthreads_or(stop);
                if (stop) {
                    if (tid == 0) atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
                    break;  // to the queue's count of CTAs done
                }
            } else {
                const uint16_t *src = reinterpret_cast<const uint16_t *>(pattern_base(pic)) +
                                      (size_t)beg.y * a.src_w + beg.x;
                // a warp per tile row, lanes along x: coalesced, and no division
                // by the runtime side
                for (int r = warp; r < side; r += WARPS)
                    for (int x = lane; x < side; x += 32) t16[r * TW + xo + x] = src[(size_t)r * a.src_w + x];
                __syncthreads();
            }
            uint32_t total = 0;  // exact, so any summation order gives the same total
            if (summed) {
#pragma unroll
                for (int w = 1; w < WARPS; ++w) total += red_u[w];
            } else {
                uint32_t acc = 0;
                for (int r = tid >> 2; r < side; r += THREADS >> 2)
                    for (int x = tid & 3; x < side; x += 4) acc += t16[r * TW + xo + x];
#pragma unroll
                for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                if (lane == 0) red_i[warp] = acc;
                __syncthreads();
#pragma unroll
                for (int w = 0; w < WARPS; ++w) total += red_i[w];
            }
            mean = (T)total / (T)(side * side);
        } else {
            const double *src = reinterpret_cast<const double *>(pattern_base(pic)) +
                                (size_t)beg.y * a.src_w + beg.x;
            double acc = 0;
            for (int i = tid; i < side * side; i += THREADS) {
                double v = src[(size_t)(i / side) * a.src_w + (i % side)];
                t64[i] = v;
                acc += v;
            }
#pragma unroll
            for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) red_s[warp] = acc;
            __syncthreads();
            double total = 0;
#pragma unroll
            for (int w = 0; w < WARPS; ++w) total += red_s[w];
            mean = (T)total / (T)(side * side);
        }

        // ---- forward rows: pairs of real rows as one complex FFT ----------
        const C *R = reinterpret_cast<const C *>(a.ref_spec) + (size_t)roi * (SL + 1) * N;
        static_assert(N / 2 <= THREADS, "one reference row sum per thread");
        // column 0 of the reference: its row sums, stored after the row FFT
        // (the load's latency hides behind it)
        const C rsum = tid < side ? __ldg(R + tid) : cmake<C>((T)0, (T)0);
        {
            const int ra = 2 * g, rb = ra + 1;
            const bool live = ra < side;  // side is even: rb < side too
            C v[E];
#pragma unroll
            for (int m = 0; m < E / 2; ++m) {
                const int x = t + G * m;
                T pa = (T)0, pb = (T)0;
                if (live && x < side) {
                    if constexpr (U16) {
                        pa = (T)t16[ra * TW + xo + x];
                        pb = (T)t16[rb * TW + xo + x];
                    } else {
                        pa = (T)t64[ra * side + x];
                        pb = (T)t64[rb * side + x];
                    }
                    pa -= mean;
                    pb -= mean;
                    pa = pa * hx[x] * hy[ra];
                    pb = pb * hx[x] * hy[rb];
                }
                v[m] = cmake<C>(pa, pb);
            }
            row_line<N, C> line{S, ra};
            group_fft<N, -1, true, T, G>(v, t, line, twf);
            const int partner = (lane & ~(G - 1)) | ((G - t) & (G - 1));
#pragma unroll
            for (int j = 0; j < E / 2; ++j) {
                C send = (t == 0) ? v[j == 0 ? 0 : E - j] : v[E - 1 - j];
                C zm = cmake<C>(__shfl_sync(0xffffffffu, send.x, partner),
                                __shfl_sync(0xffffffffu, send.y, partner));
                C z = v[j];
                const int k = t + G * j;
                if (k == 0) {
                    C zh = v[E / 2];
                    dq[ra] = dq[N + ra] = z.x;
                    dq[DQ + ra] = dq[DQ + N + ra] = zh.x;
                    dq[rb] = dq[N + rb] = z.y;
                    dq[DQ + rb] = dq[DQ + N + rb] = zh.y;
                } else {
                    C *pa = sp<N>(S, ra, k);
                    C *pb = N == 96 ? sp<N>(S, rb, k) : pa + pair_row_delta<N>(S, ra, t);
                    *pa = cmake<C>((z.x + zm.x) * (T)0.5, (z.y - zm.y) * (T)0.5);
                    *pb = cmake<C>((z.y + zm.y) * (T)0.5, (zm.x - z.x) * (T)0.5);
                }
            }
        }
        if (tid < side) {
            rs[tid] = rsum.x;
            rs[N / 2 + tid] = rsum.y;
        }
        if (queue && lead) *next_s = fetched;
        __syncthreads();
        // this CTA's next round, and this pair's successor in it (past n_pairs
        // when there is none); the one-pair form keeps the expressions that
        // compiled fastest for the 128-point kernel
        uint32_t nxt;
        if constexpr (PPC == 1) {
            nxt = queue ? *next_s : mine + stride;
            nround = queue ? nxt : round0 + stride;
        } else {
            nround = queue ? *next_s : round0 + stride;
            nxt = nround + sub;
        }
        if (nxt < a.n_pairs) beg_next = a.begins[item(nxt).y];
        // the tile is free: fetch the next pair's ROI behind the remaining passes
        if (tma && tid == 0 && nxt < a.n_pairs) issue_tile(nxt);
        if (cpa && nxt < a.n_pairs) issue_chunks(nxt);

        // ---- columns: forward FFT, conj product, inverse FFT --------------
        // Columns 1..N/2-1 by the groups (the last round leaves the last group
        // without a column); slot 0, the packed DC and Nyquist columns, is
        // packed_column's direct correlation, by every thread.
#pragma unroll 1
        for (int rnd = 0; rnd < (SL - 1 + GROUPS - 1) / GROUPS; ++rnd) {
            const int c = 1 + g + rnd * GROUPS;
            const unsigned mask = __ballot_sync(0xffffffffu, c < SL);
            if (c < SL) {
                C v[E];
#pragma unroll
                for (int m = 0; m < E / 2; ++m) v[m] = *sp<N>(S, t + G * m, c);
                col_line<N, C> line{S, c};
                if constexpr (E % 3 != 0) {
                    group_fft<N, -1, true, T, G>(v, t, line, twf, mask);
                    conj_product<N, G, T>(v, R, c, t);
                    group_fft<N, +1, false, T, G>(v, t, line, twi, mask);
                } else {
                    // Prime-factor lengths gain nothing from the zero half of
                    // the input, so both transforms run one copy of the code:
                    // the inverse as conj(forward(conj(.))).  The negations are
                    // exact, so only the pairing of multiply-adds can differ
                    // from a direct inverse.  Half the column code keeps the
                    // loop in the instruction cache.
#pragma unroll
                    for (int m = E / 2; m < E; ++m) v[m] = cmake<C>((T)0, (T)0);
#pragma unroll 1
                    for (int pass = 0; pass < 2; ++pass) {
                        group_fft<N, -1, false, T, G>(v, t, line, twf, mask);
                        if (pass == 0) {
                            conj_product<N, G, T>(v, R, c, t);
#pragma unroll
                            for (int j = 0; j < E; ++j) v[j].y = -v[j].y;
                        }
                    }
#pragma unroll
                    for (int j = 0; j < E; ++j) v[j].y = -v[j].y;
                }
#pragma unroll
                for (int j = 0; j < E; ++j) *sp<N>(S, t + G * j, c) = v[j];
            }
        }
        packed_column<N, THREADS, 2, T>([&](int tau) { return sp<N>(S, tau, 0); }, dq, rs, side, tid, 0);
        __syncthreads();

        // ---- inverse rows: pairs of half spectra -> two real rows ---------
        // Each lane scans its values in increasing map index, so a strict '>'
        // keeps the first maximum; lanes merge with the index tie-break.
        T bv = neg_inf<T>();
        uint32_t bi = 0xffffffffu;
#pragma unroll 1
        for (int rnd = 0; rnd < (N / 2) / GROUPS; ++rnd) {
            const int ra = 2 * (g + rnd * GROUPS), rb = ra + 1;
            // row rb's slots t + G j and (N - t - G j) mod N as row ra's plus a constant
            const ptrdiff_t dn = pair_row_delta<N>(S, ra, t), dk = pair_row_delta<N>(S, ra, (N - t) % SL);
            C v[E];
#pragma unroll
            for (int j = 0; j < E; ++j) {
                const int n = t + G * j;
                if (j < E / 2) {
                    const C *pa = sp<N>(S, ra, n);
                    const C ga = *pa, gb = N == 96 ? *sp<N>(S, rb, n) : pa[dn];
                    v[j] = (n == 0) ? cmake<C>(ga.x, gb.x) : cmake<C>(ga.x - gb.y, ga.y + gb.x);
                } else {
                    const int k = (n == H) ? 0 : N - n;
                    const C *pa = sp<N>(S, ra, k);
                    const C ga = *pa, gb = N == 96 ? *sp<N>(S, rb, k) : pa[dk];
                    v[j] = (n == H) ? cmake<C>(ga.y, gb.y) : cmake<C>(ga.x + gb.y, gb.x - ga.y);
                }
            }
            row_line<N, C> line{S, ra};
            group_fft<N, +1, false, T, G>(v, t, line, twi);
#pragma unroll
            for (int j = 0; j < E; ++j) *map_pair<N>(S, ra, t + G * j) = v[j];
            // map indices in increasing order: row ra, then row rb
#pragma unroll
            for (int j = 0; j < E; ++j)
                if (v[j].x > bv) {
                    bv = v[j].x;
                    bi = (uint32_t)(ra * N + t + G * j);
                }
#pragma unroll
            for (int j = 0; j < E; ++j)
                if (v[j].y > bv) {
                    bv = v[j].y;
                    bi = (uint32_t)(rb * N + t + G * j);
                }
        }

        // ---- argmax over the N x N map (maxarg.cu, first maximum) ---------
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            T ov = __shfl_xor_sync(0xffffffffu, bv, o);
            uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            better(bv, bi, ov, oi);
        }
        if (lane == 0) {
            red_v[warp] = bv;
            red_i[warp] = bi;
        }
        __syncthreads();

        // ---- neighbourhood (warp 0); the FP64 fit runs every 32 pairs ----
        if (warp == 0 && live) {
            T pv = red_v[0];
            uint32_t pk = red_i[0];
            for (int w = 1; w < WARPS; ++w) better(pv, pk, red_v[w], red_i[w]);
            if (pk >= (uint32_t)(N * N)) pk = 0;
            uint32_t mx, my;
            shift_pos(pk, POLICY_FFT, N - 1, N - 1, mx, my);
            const uint32_t slot = iter & 31;
            for (int l = lane; l < s2; l += 32) {
                uint32_t x, y;
                neighbour_pos(mx, my, l % s, l / s, s, N - 1, N - 1, x, y);
                const uint32_t q = (uint32_t)policy_index(POLICY_FFT, x, y, N - 1, N - 1);
                const uint32_t qy = q / N, qx = q % N;
                T val = reinterpret_cast<const T *>(map_pair<N>(S, (int)(qy & ~1u), (int)qx))[qy & 1];
                // an unnormalised inverse of length N scales values by N^2:
                // report them at the reference's (2*side)^2
                if (2 * side != N) val *= (T)(4 * side * side) / (T)(N * N);
                fbuf[slot * 81 + l] = val;
                if (a.neigh) reinterpret_cast<T *>(a.neigh)[(size_t)out * s2 + l] = val;
            }
            if (lane == 0) {
                // the argmax index as the reference reports it: in its own
                // 2*side map (the same index unless the ROI was zero-padded)
                uint32_t pref = pk;
                if (2 * side != N) {
                    const int ns = 2 * side, c0 = N / 2 - 1;
                    const int lx = (int)mx - c0, ly = (int)my - c0;
                    pref = (uint32_t)(((ly % ns + ns) % ns) * ns + ((lx % ns + ns) % ns));
                }
                fmeta[4 * slot] = out;
                fmeta[4 * slot + 1] = mx | (my << 16);
                fmeta[4 * slot + 2] = pref | ((uint32_t)s << 24);
                fval[slot] = 2 * side != N ? pv * ((T)(4 * side * side) / (T)(N * N)) : pv;
            }
            __syncwarp();
            const bool last = nxt >= a.n_pairs;
            if (slot == 31 || last) fit_batch<T>(a, fbuf, fmeta, fval, (int)slot + 1, lane, N - 1);
        }
        const bool ahead = sum_ahead && nxt < a.n_pairs;
        if (ahead && warp != 0) {
            // the next tile was requested after this pair's row pass: wait for it
            // and sum it over the other warps' threads
            if (!mbar_wait(bar, (iter + 1) & 1)) atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
            const int nxo = (int)(beg_next.x & 7u);
            const int u = tid - 32;
            uint32_t acc = 0;
            for (int r = u >> 2; r < side; r += (THREADS - 32) >> 2)
                for (int x = u & 3; x < side; x += 4) acc += t16[r * TW + nxo + x];
#pragma unroll
            for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0) red_u[warp] = acc;
        }
        summed = ahead;
        __syncthreads();
    }
    if (queue && lead) {
        // every CTA has taken its last round from the queue before it counts
        // itself done, so the last one can zero the queue for the next launch
        __threadfence();
        if (atomicAdd(queue + 1, 1u) == gridDim.x - 1) {
            atomicExch(queue, 0u);
            atomicExch(queue + 1, 0u);
        }
    }
}


// ---- 256-point transforms on a cluster of two CTAs ---------------------------
// An FP32 256 x 128 half spectrum is 256 KB, more than one CTA's shared memory.
// The two CTAs of a cluster split it by slots -- CTA r holds slots 64r..64r+63
// of every spectrum row -- and exchange through distributed shared memory:
//   sums          each CTA sums its half of the ROI rows; the partial sums cross;
//   row pass      CTA r transforms ROI rows 64r..64r+63 (TMA box of 64 rows) and
//                 writes every output slot into the CTA that owns it;
//   column pass   local: forward FFT, conj product, inverse FFT of its 64 columns;
//   inverse rows  CTA r produces map rows 128r..128r+127, reading the partner's
//                 64 slots of each row; the real map goes back over the same
//                 two rows, map rows (2p, 2p+1) at column x as one slot: slot
//                 x mod 128 of row 2p (x < 128) or 2p+1, in its owner CTA;
//   peak, fit     CTA 0 merges both maxima, reads the neighbourhood from either
//                 CTA and runs the batched FP64 fit.
// Every thread of both CTAs passes the same cluster barriers in every pair and
// none leaves the loop early, so a barrier cannot wait on a missing CTA; a TMA
// wait that runs out only flags the error.
namespace cl {

constexpr int N = 256, G = 16, E = N / G, H = N / 2;
constexpr int SLOTS = N / 4;        // slots of each spectrum row held per CTA
constexpr int GROUPS = 16, THREADS = GROUPS * G, WARPS = THREADS / 32;
constexpr int ROWS = H / 2;         // ROI rows staged per CTA

template <typename C> __device__ __forceinline__ C *csp(C *S, int row, int slot)
{
    // XOR by the row's low 4 bits: a 16-lane group's column access (rows t + 16m)
    // and row access (16 consecutive slots) both hit 16 distinct bank pairs
    return S + row * SLOTS + (slot ^ (row & 15));
}

constexpr size_t up(size_t v, size_t a) { return (v + a - 1) / a * a; }

struct layout {
    static constexpr size_t spectrum = 0;                               // N x SLOTS float2
    static constexpr size_t xch = spectrum + (size_t)N * SLOTS * 8;     // GROUPS x N float2
    static constexpr size_t tw_fwd = xch + (size_t)GROUPS * N * 8;
    static constexpr size_t tw_bytes = (size_t)G * tw_stride<N, G, float2>() * 8;  // [G][TS]
    static constexpr size_t tw_inv = tw_fwd + tw_bytes;
    static constexpr size_t hann = tw_inv + tw_bytes;                   // hx[side], hy[side]
    static constexpr size_t dq = hann + (size_t)N * 4;                  // DC, Nyquist lines
    static constexpr size_t rsum = dq + (size_t)2 * packed_dq<N>() * 4;  // reference row sums
    static constexpr size_t red_val = rsum + (size_t)N * 4;
    static constexpr size_t red_idx = red_val + 32 * 4;
    static constexpr size_t psum = red_idx + 32 * 4;                    // partial sums [2]
    static constexpr size_t pbest_v = psum + 16;                        // CTA maxima [2]
    static constexpr size_t pbest_i = pbest_v + 16;
    static constexpr size_t barrier = pbest_i + 16;                     // mbarrier, next pair
    static constexpr size_t fit_vals = barrier + 16;
    static constexpr size_t fit_meta = fit_vals + 32 * 81 * 4;
    static constexpr size_t fit_peak = fit_meta + 32 * 4 * 4;
    static constexpr size_t tile = up(fit_peak + 32 * 4, 128);
    static constexpr size_t bytes = tile + (size_t)ROWS * (H + 8) * 2;
};
static_assert(layout::bytes <= 227 * 1024, "cluster layout must fit one CTA's shared memory");

}  // namespace cl

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(cl::THREADS, 1)
    fused_cluster_kernel(const fused_args a, const __grid_constant__ CUtensorMap tmap)
{
    namespace cg = cooperative_groups;
    using namespace cl;
    using T = float;
    using C = cplx<T>;
    using L = cl::layout;
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank(), peer = rank ^ 1;
    const uint32_t clusters = gridDim.x / 2, cid = blockIdx.x / 2;
    const int side = a.side;
    const int TW = (side + 14) & ~7;

    extern __shared__ __align__(1024) unsigned char smem[];
    C *S = reinterpret_cast<C *>(smem + L::spectrum);
    C *Sp = cluster.map_shared_rank(S, peer);
    C *X = reinterpret_cast<C *>(smem + L::xch);
    C *twf = reinterpret_cast<C *>(smem + L::tw_fwd);
    C *twi = reinterpret_cast<C *>(smem + L::tw_inv);
    T *hx = reinterpret_cast<T *>(smem + L::hann);
    T *hy = hx + side;
    constexpr int DQ = packed_dq<N>();
    T *dq = reinterpret_cast<T *>(smem + L::dq);        // DC and Nyquist outputs of both CTAs' rows
    T *dq_p = cluster.map_shared_rank(dq, peer);
    T *rs = reinterpret_cast<T *>(smem + L::rsum);      // the reference's row sums (this ROI)
    T *red_v = reinterpret_cast<T *>(smem + L::red_val);
    uint32_t *red_i = reinterpret_cast<uint32_t *>(smem + L::red_idx);
    uint32_t *psum = reinterpret_cast<uint32_t *>(smem + L::psum);
    uint32_t *psum_p = cluster.map_shared_rank(psum, peer);
    T *pbest_v = reinterpret_cast<T *>(smem + L::pbest_v);
    uint32_t *pbest_i = reinterpret_cast<uint32_t *>(smem + L::pbest_i);
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + L::barrier);
    // the pair queue: CTA 0's thread 0 takes the cluster's next pair and puts
    // it in both CTAs' word after the mbarrier
    uint32_t *const queue = a.pair_queue;
    uint32_t *next_s = reinterpret_cast<uint32_t *>(smem + L::barrier + 8);
    uint32_t *next_p = cluster.map_shared_rank(next_s, peer);
    T *fbuf = reinterpret_cast<T *>(smem + L::fit_vals);
    uint32_t *fmeta = reinterpret_cast<uint32_t *>(smem + L::fit_meta);
    T *fval = reinterpret_cast<T *>(smem + L::fit_peak);
    uint16_t *t16 = reinterpret_cast<uint16_t *>(smem + L::tile);

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int t = lane & (G - 1), g = tid / G;
    C *xg = X + g * N;  // this group's exchange line
    struct xline {
        C *p;
        __device__ __forceinline__ C *operator()(int q) const { return p + q; }
    };
    const xline xl{xg};
    // owner of slot k (0..127) of a spectrum row
    auto owner = [&](int k) -> C * { return (k >> 6) == rank ? S : Sp; };

    const C *gtw = reinterpret_cast<const C *>(a.twiddles);
    constexpr int TS = tw_stride<N, G, C>();
    for (int i = tid; i < G * TS; i += THREADS) {
        const int k1 = i % TS;
        const C w = k1 < E ? gtw[(i / TS) * k1] : cmake<C>((T)0, (T)0);
        twf[i] = w;
        twi[i] = cconj(w);
    }
    const T *ghann = reinterpret_cast<const T *>(a.hann);
    for (int i = tid; i < 2 * side; i += THREADS) hx[i] = ghann[i];
    // the zero padding of the DC and Nyquist lines (the rows pass writes rows
    // 0..N/2-1 and their copy at N..3N/2-1, in both CTAs)
    for (int i = tid; i < 2 * DQ; i += THREADS) {
        const int y = i % DQ;
        if ((y >= N / 2 && y < N) || y >= 3 * N / 2) dq[i] = (T)0;
    }
    const bool tma = a.stage == STAGE_TMA;
    if (tid == 0) {
        mbar_init(bar, 1);
        fence_proxy_async();
    }
    __syncthreads();

    auto item = [&](uint32_t pair) -> uint4 {
        if (a.items) return a.items[pair];
        return make_uint4(pair / a.n_rois, pair % a.n_rois, pair, (uint32_t)a.fitsize);
    };
    auto pattern_base = [&](uint32_t pic) -> const uint16_t * {
        if (a.pattern_ptrs) return reinterpret_cast<const uint16_t *>(a.pattern_ptrs[pic]);
        return reinterpret_cast<const uint16_t *>(a.pics) + (size_t)pic * a.src_w * a.src_h;
    };
    auto issue_tile = [&](uint32_t pair) {
        const uint4 it = item(pair);
        const uint2 b = a.begins[it.y];
        fence_proxy_async();
        mbar_expect_tx(bar, TW * ROWS * 2);
        tma_load_3d(t16, &tmap, (int)(b.x & ~7u), (int)b.y + ROWS * rank, (int)it.x, bar);
    };
    if (tma && tid == 0 && cid < a.n_pairs) issue_tile(cid);

    uint32_t iter = 0;
    for (uint32_t pair = cid, npair = 0; pair < a.n_pairs; pair = npair, ++iter) {
        // the queue's answer is needed after the row pass, which hides its latency
        uint32_t fetched = 0;
        if (queue && rank == 0 && tid == 0) fetched = atomicAdd(queue, 1u) + clusters;
        const uint4 it = item(pair);
        const uint32_t pic = it.x, roi = it.y, out = it.z;
        const int s = (int)it.w, s2 = s * s;
        const uint2 beg = a.begins[roi];
        const int xo = (int)(beg.x & 7u);
        const int r0 = ROWS * rank;                      // first ROI row of this CTA
        const int nrows = max(0, min(ROWS, side - r0));  // live ROI rows of this CTA

        // ---- this CTA's half of the ROI, its partial sum -------------------
        if (tma) {
            if (!mbar_wait(bar, iter & 1) && tid == 0) atomicOr(a.err, DEV_ERR_TMA_TIMEOUT);
        } else {
            const uint16_t *src = pattern_base(pic) + (size_t)(beg.y + r0) * a.src_w + beg.x;
            for (int r = warp; r < nrows; r += WARPS)
                for (int x = lane; x < side; x += 32) t16[r * TW + xo + x] = src[(size_t)r * a.src_w + x];
            __syncthreads();
        }
        uint32_t acc = 0;
        for (int r = tid >> 2; r < nrows; r += THREADS >> 2)
            for (int x = tid & 3; x < side; x += 4) acc += t16[r * TW + xo + x];
#pragma unroll
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) red_i[warp] = acc;
        __syncthreads();
        if (tid == 0) {
            uint32_t part = 0;
            for (int w = 0; w < WARPS; ++w) part += red_i[w];
            psum[rank] = part;
            psum_p[rank] = part;
        }
        // B0: both partial sums are in place, and the previous pair's reads of
        // the partner's map are finished
        cluster.sync();
        const T mean = (T)(psum[0] + psum[1]) / (T)(side * side);

        // ---- forward rows: pairs of real rows as one complex FFT -----------
        const C *R = reinterpret_cast<const C *>(a.ref_spec) + (size_t)roi * (H + 1) * N;
        static_assert(N / 2 <= THREADS, "one reference row sum per thread");
        // column 0 of the reference: its row sums, stored after the row FFTs
        const C rsum = tid < side ? __ldg(R + tid) : cmake<C>((T)0, (T)0);
#pragma unroll 1
        for (int rnd = 0; rnd < ROWS / 2 / GROUPS; ++rnd) {
            const int rl = 2 * (g + GROUPS * rnd), ra = r0 + rl, rb = ra + 1;
            const bool live = ra < side;
            C v[E];
#pragma unroll
            for (int m = 0; m < E / 2; ++m) {
                const int x = t + G * m;
                T pa = (T)0, pb = (T)0;
                if (live && x < side) {
                    pa = ((T)t16[rl * TW + xo + x] - mean) * hx[x] * hy[ra];
                    pb = ((T)t16[(rl + 1) * TW + xo + x] - mean) * hx[x] * hy[rb];
                }
                v[m] = cmake<C>(pa, pb);
            }
            group_fft<N, -1, true, T, G>(v, t, xl, twf);
            const int partner = (lane & ~(G - 1)) | ((G - t) & (G - 1));
#pragma unroll
            for (int j = 0; j < E / 2; ++j) {
                C send = (t == 0) ? v[j == 0 ? 0 : E - j] : v[E - 1 - j];
                C zm = cmake<C>(__shfl_sync(0xffffffffu, send.x, partner),
                                __shfl_sync(0xffffffffu, send.y, partner));
                C z = v[j];
                const int k = t + G * j;
                C *D = owner(k);
                if (k == 0) {
                    // the DC and Nyquist outputs go to both CTAs' lines
                    C zh = v[E / 2];
                    for (T *line : {dq, dq_p}) {
                        line[ra] = line[N + ra] = z.x;
                        line[DQ + ra] = line[DQ + N + ra] = zh.x;
                        line[rb] = line[N + rb] = z.y;
                        line[DQ + rb] = line[DQ + N + rb] = zh.y;
                    }
                } else {
                    *csp(D, ra, k & 63) = cmake<C>((z.x + zm.x) * (T)0.5, (z.y - zm.y) * (T)0.5);
                    *csp(D, rb, k & 63) = cmake<C>((z.y + zm.y) * (T)0.5, (zm.x - z.x) * (T)0.5);
                }
            }
        }
        if (tid < side) {
            rs[tid] = rsum.x;
            rs[N / 2 + tid] = rsum.y;
        }
        if (queue && rank == 0 && tid == 0) {
            *next_s = fetched;
            *next_p = fetched;
        }
        __syncthreads();
        if (!queue && tma && tid == 0 && pair + clusters < a.n_pairs) issue_tile(pair + clusters);
        cluster.sync();  // B1: every spectrum row and both DC/Nyquist lines are complete
        // the cluster's next pair (past n_pairs when there is none); with a
        // queue, this CTA's half of its ROI is requested now
        npair = queue ? *next_s : pair + clusters;
        if (queue && tma && tid == 0 && npair < a.n_pairs) issue_tile(npair);

        // ---- columns: forward FFT, conj product, inverse FFT (local) -------
        // CTA 0's slot 0 packs the DC and Nyquist columns: it is the direct
        // correlation of packed_column, CTA 0 the DC half and CTA 1 the
        // Nyquist half; CTA 0's groups take its columns 1..63 (the last round
        // leaves its last group without one), CTA 1's groups all 64 of theirs.
        const int c_first = rank == 0 ? 1 : 0;
#pragma unroll 1
        for (int rnd = 0; rnd < SLOTS / GROUPS; ++rnd) {
            const int c = c_first + g + rnd * GROUPS, kx = SLOTS * rank + c;
            const unsigned mask = __ballot_sync(0xffffffffu, c < SLOTS);
            if (c < SLOTS) {
                C v[E];
#pragma unroll
                for (int m = 0; m < E / 2; ++m) v[m] = *csp(S, t + G * m, c);
                struct cline {
                    C *S;
                    int c;
                    __device__ __forceinline__ C *operator()(int q) const { return csp(S, q, c); }
                } line{S, c};
                group_fft<N, -1, true, T, G>(v, t, line, twf, mask);
                const C *Rc = R + (size_t)kx * N;
#pragma unroll
                for (int j = 0; j < E; ++j) v[j] = cmulc(v[j], __ldg(Rc + t + G * j));
                group_fft<N, +1, false, T, G>(v, t, line, twi, mask);
#pragma unroll
                for (int j = 0; j < E; ++j) *csp(S, t + G * j, c) = v[j];
            }
        }
        C *S0 = owner(0);  // CTA 0's spectrum, which holds slot 0
        packed_column<N, THREADS, 1, T>([&](int tau) { return csp(S0, tau, 0); }, dq, rs, side, tid, rank);
        cluster.sync();  // B2: every column is back in the spectrum

        // ---- inverse rows 128r..128r+127: two Hermitian rows per FFT -------
        T bv = neg_inf<T>();
        uint32_t bi = 0xffffffffu;
#pragma unroll 1
        for (int rnd = 0; rnd < H / 2 / GROUPS; ++rnd) {
            const int ra = H * rank + 2 * (g + GROUPS * rnd), rb = ra + 1;
            C v[E];
#pragma unroll
            for (int j = 0; j < E; ++j) {
                const int n = t + G * j;
                if (j < E / 2) {
                    C *D = owner(n);
                    C ga = *csp(D, ra, n & 63), gb = *csp(D, rb, n & 63);
                    v[j] = (n == 0) ? cmake<C>(ga.x, gb.x) : cmake<C>(ga.x - gb.y, ga.y + gb.x);
                } else {
                    const int k = (n == H) ? 0 : N - n;
                    C *D = owner(k);
                    C ga = *csp(D, ra, k & 63), gb = *csp(D, rb, k & 63);
                    v[j] = (n == H) ? cmake<C>(ga.y, gb.y) : cmake<C>(ga.x + gb.y, gb.x - ga.y);
                }
            }
            group_fft<N, +1, false, T, G>(v, t, xl, twi);
            // map rows ra and rb at column x as one slot: slot x mod 128 of
            // spectrum row ra (x < 128) or rb, in the CTA that owns that slot
#pragma unroll
            for (int j = 0; j < E; ++j) {
                const int x = t + G * j, q = x & (H - 1);
                *csp(owner(q), ra + (x >= H), q & 63) = v[j];
            }
            // map indices in increasing order: row ra, then row rb
#pragma unroll
            for (int j = 0; j < E; ++j)
                if (v[j].x > bv) {
                    bv = v[j].x;
                    bi = (uint32_t)(ra * N + t + G * j);
                }
#pragma unroll
            for (int j = 0; j < E; ++j)
                if (v[j].y > bv) {
                    bv = v[j].y;
                    bi = (uint32_t)(rb * N + t + G * j);
                }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            T ov = __shfl_xor_sync(0xffffffffu, bv, o);
            uint32_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
            better(bv, bi, ov, oi);
        }
        if (lane == 0) {
            red_v[warp] = bv;
            red_i[warp] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            T cv = red_v[0];
            uint32_t ci = red_i[0];
            for (int w = 1; w < WARPS; ++w) better(cv, ci, red_v[w], red_i[w]);
            // both CTAs' maxima meet in CTA 0
            *cluster.map_shared_rank(pbest_v + rank, 0) = cv;
            *cluster.map_shared_rank(pbest_i + rank, 0) = ci;
        }
        cluster.sync();  // B3: the map and both maxima are in place

        // ---- neighbourhood and fit (CTA 0, warp 0) -------------------------
        if (rank == 0 && warp == 0) {
            T pv = pbest_v[0];
            uint32_t pk = pbest_i[0];
            better(pv, pk, pbest_v[1], pbest_i[1]);
            if (pk >= (uint32_t)(N * N)) pk = 0;
            uint32_t mx, my;
            shift_pos(pk, POLICY_FFT, N - 1, N - 1, mx, my);
            const uint32_t slot = iter & 31;
            const T scale = (T)(4 * side * side) / (T)(N * N);
            for (int l = lane; l < s2; l += 32) {
                uint32_t x, y;
                neighbour_pos(mx, my, l % s, l / s, s, N - 1, N - 1, x, y);
                const uint32_t qm = (uint32_t)policy_index(POLICY_FFT, x, y, N - 1, N - 1);
                const int qy = (int)(qm / N), qx = (int)(qm % N), q = qx & (H - 1);
                T val = reinterpret_cast<const T *>(csp(owner(q), (qy & ~1) + (qx >= H), q & 63))[qy & 1];
                if (2 * side != N) val *= scale;
                fbuf[slot * 81 + l] = val;
                if (a.neigh) reinterpret_cast<T *>(a.neigh)[(size_t)out * s2 + l] = val;
            }
            if (lane == 0) {
                uint32_t pref = pk;
                if (2 * side != N) {
                    const int ns = 2 * side, c0 = N / 2 - 1;
                    const int lx = (int)mx - c0, ly = (int)my - c0;
                    pref = (uint32_t)(((ly % ns + ns) % ns) * ns + ((lx % ns + ns) % ns));
                }
                fmeta[4 * slot] = out;
                fmeta[4 * slot + 1] = mx | (my << 16);
                fmeta[4 * slot + 2] = pref | ((uint32_t)s << 24);
                fval[slot] = 2 * side != N ? pv * scale : pv;
            }
            __syncwarp();
            const bool last = npair >= a.n_pairs;
            if (slot == 31 || last) fit_batch<T>(a, fbuf, fmeta, fval, (int)slot + 1, lane, N - 1);
        }
        __syncthreads();
    }
    // the partner may still read this CTA's shared memory: leave together
    cluster.sync();
    if (queue && rank == 0 && tid == 0) {
        // every cluster has taken its last pair before it counts itself done
        __threadfence();
        if (atomicAdd(queue + 1, 1u) == clusters - 1) {
            atomicExch(queue, 0u);
            atomicExch(queue + 1, 0u);
        }
    }
}

static cudaError_t launch_cluster(const fused_args &a, const CUtensorMap *tmap, int grid, cudaStream_t st)
{
    auto k = fused_cluster_kernel;
    const size_t smem = cl::layout::bytes;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (grid <= 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        grid += sms;  // one CTA per SM, two per cluster, less the CTAs left free
        if (grid < 2) grid = 2;
    }
    grid &= ~1;
    if ((uint32_t)grid > 2 * a.n_pairs) grid = (int)(2 * a.n_pairs);
    if (grid < 2) return cudaSuccess;
    k<<<grid, cl::THREADS, smem, st>>>(a, *tmap);
    return cudaGetLastError();
}

template <int N, int G, typename T, typename IN, int PPC = fused_pairs_per_cta<N, T>()>
static cudaError_t launch_one(const fused_args &a, const CUtensorMap *tmap, int grid,
                              cudaStream_t st)
{
    auto k = fused_fft_kernel<N, G, T, IN, PPC>;
    constexpr int ppc = PPC;
    constexpr int threads = N * G / 4 * ppc;
    const size_t smem = fused_layout<N, G, T, PPC>::bytes;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    if (grid <= 0) {
        int per_sm = 0, dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem);
        if (e != cudaSuccess) return e;
        if (per_sm < 1) per_sm = 1;
        // The FP32 128-point kernel holds 2 pairs per SM; without a pair queue,
        // three waves of CTAs (each with a third of the pairs) end more evenly
        // than one when every CTA still gets 16 pairs or more (25,600 pairs:
        // 1.206 against 1.225 ms).  With a queue one wave ends more evenly still
        // (1.166 ms).  Launches that leave CTA slots free (grid < 0) keep one wave.
        const int waves = grid == 0 && !a.pair_queue && N == 128 && sizeof(T) == 4 &&
                                  a.n_pairs >= 3u * 16u * (uint32_t)(per_sm * sms)
                              ? 3
                              : 1;
        grid += waves * per_sm * sms;  // less the CTAs left free
        if (grid < 1) grid = 1;
    }
    const uint32_t rounds = (a.n_pairs + ppc - 1) / ppc;  // CTAs with a pair to start on
    if ((uint32_t)grid > rounds) grid = (int)rounds;
    if (grid < 1) return cudaSuccess;
    k<<<grid, threads, smem, st>>>(a, *tmap);
    return cudaGetLastError();
}

bool fused_supported(uint32_t fft_n, bool dbl, bool in_f64)
{
    return fft_n == 64 || fft_n == 96 || fft_n == 128 || (fft_n == 192 && !dbl) ||
           (fft_n == 256 && !dbl && !in_f64);
}

uint32_t fused_size_for(uint32_t side, bool dbl, bool in_f64)
{
    for (uint32_t n : {64u, 96u, 128u, 192u, 256u})
        if (2 * side <= n && fused_supported(n, dbl, in_f64)) return n;
    return 0;
}

cudaError_t preload_fused(uint32_t fft_n, bool dbl, bool in_f64)
{
    // the launcher sets the kernel's shared-memory attribute (which loads its
    // module) and then has no pairs to launch
    fused_args a{};
    CUtensorMap map;
    std::memset(&map, 0, sizeof map);
    return launch_fused(fft_n, dbl, in_f64, a, &map, 0, 0);
}

size_t fused_smem_bytes(uint32_t fft_n, bool dbl)
{
    switch (fft_n) {
    case 64: return dbl ? fused_layout<64, 8, double>::bytes : fused_layout<64, 8, float>::bytes;
    case 96: return dbl ? fused_layout<96, 4, double>::bytes : fused_layout<96, 4, float>::bytes;
    case 128: return dbl ? fused_layout<128, 8, double>::bytes : fused_layout<128, 8, float>::bytes;
    case 192: return fused_layout<192, 8, float>::bytes;
    case 256: return cl::layout::bytes;
    default: return 0;
    }
}

uint32_t fused_box_rows(uint32_t fft_n, uint32_t side)
{
    return fft_n == 256 ? cl::ROWS : side;
}

template <int N, int G>
static cudaError_t launch_n(bool dbl, bool in_f64, const fused_args &a, const CUtensorMap *tmap,
                            int grid, cudaStream_t st)
{
    if (dbl)
        return in_f64 ? launch_one<N, G, double, double>(a, tmap, grid, st)
                      : launch_one<N, G, double, uint16_t>(a, tmap, grid, st);
    if (in_f64) return launch_one<N, G, float, double>(a, tmap, grid, st);
    if constexpr (N == 96) {
        // 1, 2 or 4 pairs per CTA.  The default is 2 with a pair queue (two
        // CTAs per SM; side 48: 33.0 against 32.4 M pairs/s with 4) and 4
        // without one, where a single CTA per SM ends a fixed walk more evenly
        if (a.pairs_per_cta == 1) return launch_one<N, G, float, uint16_t, 1>(a, tmap, grid, st);
        if (a.pairs_per_cta == 2 || (a.pairs_per_cta == 0 && a.pair_queue))
            return launch_one<N, G, float, uint16_t, 2>(a, tmap, grid, st);
    }
    return launch_one<N, G, float, uint16_t>(a, tmap, grid, st);
}

cudaError_t launch_fused(uint32_t fft_n, bool dbl, bool in_f64, const fused_args &a,
                         const CUtensorMap *tmap, int grid, cudaStream_t st)
{
    if (!fused_supported(fft_n, dbl, in_f64)) return cudaErrorInvalidValue;
    if (fft_n == 256) return launch_cluster(a, tmap, grid, st);
    switch (fft_n) {
    case 64: return launch_n<64, 8>(dbl, in_f64, a, tmap, grid, st);
    case 96: return launch_n<96, 4>(dbl, in_f64, a, tmap, grid, st);
    case 128: return launch_n<128, 8>(dbl, in_f64, a, tmap, grid, st);
    default: break;
    }
    // 192 points, FP32 only (an FP64 spectrum would not fit in shared memory)
    return in_f64 ? launch_one<192, 8, float, double>(a, tmap, grid, st)
                  : launch_one<192, 8, float, uint16_t>(a, tmap, grid, st);
}

}  // namespace emida_gb
