// fft.cuh -- register/shared-memory FFT building blocks for sm_103a.
//
// These replace the cuFFT R2C/C2R calls of the reference
// (src/gpu_offset.hpp:171-183, :303-316, src/cufft_helpers.hpp:105-155).
//
// One 1-D transform of length N = 8*E is carried by a group of 8 consecutive
// lanes of one warp ("fft group"); each lane holds E complex values.  Lane t of
// the group holds element n = t + 8*j in register j, both before and after the
// transform (the scheme is self-sorting), so transforms chain without
// permutations.  The only exchange goes through shared memory inside the
// group's own 128-slot line and needs __syncwarp only.
//
//   n = t + 8m, k = k1 + E*k2:
//   X[k1 + E k2] = sum_t W8^{t k2} * W_N^{t k1} * sum_m x[t + 8m] W_E^{m k1}
//   pass 1: E-point DFT over m in registers; twiddle W_N^{t k1};
//   exchange; pass 2: E/8 8-point DFTs over t.
#pragma once

#include "common.cuh"

namespace emida_gb {

template <typename T> struct cplx_t;
template <> struct cplx_t<float> { using type = float2; };
template <> struct cplx_t<double> { using type = double2; };

template <typename T> using cplx = typename cplx_t<T>::type;

template <typename C> __device__ __forceinline__ C cmake(decltype(C::x) x, decltype(C::x) y)
{
    C c;
    c.x = x;
    c.y = y;
    return c;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return cmake<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return cmake<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b)
{
    return cmake<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename C> __device__ __forceinline__ C cmulc(C a, C b)
{
    return cmake<C>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename C> __device__ __forceinline__ C cconj(C a) { return cmake<C>(a.x, -a.y); }

// cos/sin(2*pi*k/16), k = 0..7, correctly rounded decimal expansions.
__device__ __forceinline__ double c16(int k)
{
    switch (k & 15) {
    case 0: return 1.0;
    case 1: return 0.92387953251128675613;
    case 2: return 0.70710678118654752440;
    case 3: return 0.38268343236508977173;
    case 4: return 0.0;
    case 5: return -0.38268343236508977173;
    case 6: return -0.70710678118654752440;
    case 7: return -0.92387953251128675613;
    default: return -c16(k - 8);
    }
}
__device__ __forceinline__ double s16(int k) { return c16(k - 4); }

// Multiply a by W_16^k, W = exp(DIR * 2 pi i / 16), DIR = -1 forward, +1 inverse.
// k is a compile-time constant after unrolling; exact cases are special-cased.
template <int DIR, typename C> __device__ __forceinline__ C tw16(C a, int k)
{
    using T = decltype(C::x);
    k &= 15;
    if (k == 0) return a;
    if (k == 8) return cmake<C>(-a.x, -a.y);
    if (k == 4) return DIR < 0 ? cmake<C>(a.y, -a.x) : cmake<C>(-a.y, a.x);
    if (k == 12) return DIR < 0 ? cmake<C>(-a.y, a.x) : cmake<C>(a.y, -a.x);
    T c = (T)c16(k);
    T s = (T)(DIR * s16(k));
    return cmake<C>(a.x * c - a.y * s, a.x * s + a.y * c);
}

// In-register DFT of length L (power of two <= 16), natural order in and out.
// Radix-2 decimation in frequency, recursively.
template <int L, int DIR, typename C> struct rdft {
    static __device__ __forceinline__ void run(C *a)
    {
        C e[L / 2], o[L / 2];
#pragma unroll
        for (int n = 0; n < L / 2; ++n) {
            e[n] = cadd(a[n], a[n + L / 2]);
            o[n] = tw16<DIR>(csub(a[n], a[n + L / 2]), n * (16 / L));
        }
        rdft<L / 2, DIR, C>::run(e);
        rdft<L / 2, DIR, C>::run(o);
#pragma unroll
        for (int k = 0; k < L / 2; ++k) {
            a[2 * k] = e[k];
            a[2 * k + 1] = o[k];
        }
    }
    // Same transform when a[L/2 .. L-1] are known to be zero.
    static __device__ __forceinline__ void run_half(C *a)
    {
        C e[L / 2], o[L / 2];
#pragma unroll
        for (int n = 0; n < L / 2; ++n) {
            e[n] = a[n];
            o[n] = tw16<DIR>(a[n], n * (16 / L));
        }
        rdft<L / 2, DIR, C>::run(e);
        rdft<L / 2, DIR, C>::run(o);
#pragma unroll
        for (int k = 0; k < L / 2; ++k) {
            a[2 * k] = e[k];
            a[2 * k + 1] = o[k];
        }
    }
};
template <int DIR, typename C> struct rdft<1, DIR, C> {
    static __device__ __forceinline__ void run(C *) {}
    static __device__ __forceinline__ void run_half(C *) {}
};

// Shared-memory view of one transform line of N complex slots.  The group
// passes an accessor that maps a line position (0..N-1) to a slot pointer.
// Exchange position of A'[t][k1]: 8*k1 + ((t + k1) & 7), chosen so that both
// the writes (fixed k1) and the reads (fixed t) of the eight lanes fall in
// eight different rows / slots.
// tw: the inter-pass twiddles of this direction laid out [k1][lane]:
// tw[8*k1 + t] = W_N^{t*k1} (exp(-2 pi i t k1 / N) forward, its conjugate
// inverse), so the eight lanes of a group read eight consecutive slots.
template <int N, int DIR, bool HALF_INPUT, typename T, typename Line>
__device__ __forceinline__ void group_fft(cplx<T> *v, int t, const Line &line,
                                          const cplx<T> *__restrict__ tw)
{
    using C = cplx<T>;
    constexpr int E = N / 8;
    static_assert(E == 8 || E == 16, "group_fft supports N = 64 and N = 128");
    if (HALF_INPUT)
        rdft<E, DIR, C>::run_half(v);
    else
        rdft<E, DIR, C>::run(v);
#pragma unroll
    for (int k1 = 1; k1 < E; ++k1) v[k1] = cmul(v[k1], tw[8 * k1 + t]);
    __syncwarp();
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) *line(8 * k1 + ((t + k1) & 7)) = v[k1];
    __syncwarp();
    // pass 2: for i in [0, E/8): k1 = t + 8 i, DFT over the 8 lanes' values
#pragma unroll
    for (int i = 0; i < E / 8; ++i) {
        C a[8];
#pragma unroll
        for (int s = 0; s < 8; ++s) a[s] = *line(8 * t + 64 * i + ((s + t) & 7));
        rdft<8, DIR, C>::run(a);
#pragma unroll
        for (int k2 = 0; k2 < 8; ++k2) v[i + (E / 8) * k2] = a[k2];
    }
    __syncwarp();
}

}  // namespace emida_gb
