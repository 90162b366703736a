// fft.cuh -- register/shared-memory FFT building blocks for sm_103a.
//
// These replace the cuFFT R2C/C2R calls of the reference
// (src/gpu_offset.hpp:171-183, :303-316, src/cufft_helpers.hpp:105-155).
//
// One 1-D transform of length N = G*E is carried by a group of G = 4 or 8
// consecutive lanes of one warp ("fft group"); each lane holds E complex
// values.  Lane t of the group holds element n = t + G*j in register j, both
// before and after the transform (the scheme is self-sorting), so transforms
// chain without permutations.  The only exchange goes through shared memory
// inside the group's own line of N slots and needs __syncwarp only.
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

// cos(2*pi*k/48) for k = 0..12 (first quadrant), 25 significant digits; the
// other quadrants follow by symmetry.  Every register DFT length used here
// (2, 3, 4, 6, 8, 12, 16, 24) divides 48.
__device__ __forceinline__ double c48(int k)
{
    k %= 48;
    if (k < 0) k += 48;
    if (k > 24) k = 48 - k;            // cos(-x) = cos(x)
    const bool neg = k > 12;
    if (neg) k = 24 - k;               // cos(pi - x) = -cos(x)
    double v;
    switch (k) {
    case 0: v = 1.0; break;
    case 1: v = 0.9914448613738104111445575; break;
    case 2: v = 0.9659258262890682867497432; break;
    case 3: v = 0.9238795325112867561281832; break;
    case 4: v = 0.8660254037844386467637232; break;
    case 5: v = 0.7933533402912351645797770; break;
    case 6: v = 0.7071067811865475244008444; break;
    case 7: v = 0.6087614290087206394160975; break;
    case 8: v = 0.5; break;
    case 9: v = 0.3826834323650897717284600; break;
    case 10: v = 0.2588190451025207623488988; break;
    case 11: v = 0.1305261922200515915484062; break;
    default: v = 0.0; break;
    }
    return neg ? -v : v;
}
__device__ __forceinline__ double s48(int k) { return c48(k - 12); }

// Multiply a by W_L^n, W = exp(DIR * 2 pi i / L), DIR = -1 forward, +1 inverse,
// L dividing 48.  n and L are compile-time constants after unrolling; the
// quarter turns are exact.
template <int DIR, typename C> __device__ __forceinline__ C twl(C a, int n, int L)
{
    using T = decltype(C::x);
    int k = (n * (48 / L)) % 48;
    if (k == 0) return a;
    if (k == 24) return cmake<C>(-a.x, -a.y);
    if (k == 12) return DIR < 0 ? cmake<C>(a.y, -a.x) : cmake<C>(-a.y, a.x);
    if (k == 36) return DIR < 0 ? cmake<C>(-a.y, a.x) : cmake<C>(a.y, -a.x);
    T c = (T)c48(k);
    T s = (T)(DIR * s48(k));
    return cmake<C>(a.x * c - a.y * s, a.x * s + a.y * c);
}

// In-register DFT of length L (2^a * 3^b <= 24), natural order in and out:
// radix-2 decimation in frequency down to length 3 or 1.
template <int L, int DIR, typename C> struct rdft {
    static __device__ __forceinline__ void run(C *a)
    {
        C e[L / 2], o[L / 2];
#pragma unroll
        for (int n = 0; n < L / 2; ++n) {
            e[n] = cadd(a[n], a[n + L / 2]);
            o[n] = twl<DIR>(csub(a[n], a[n + L / 2]), n, L);
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
            o[n] = twl<DIR>(a[n], n, L);
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
// Lengths 3 * M with M = 2, 4, 8 (6, 12, 24): the Good-Thomas prime-factor
// algorithm, which needs no twiddles between its 3-point and M-point passes.
// Input n = (M n1 + 3 n2) mod L goes to row n1 (3-point DFTs along n1), and
// output k = (A k1 + B k2) mod L comes from k1 of the 3-point pass and k2 of
// the M-point pass, A = M (M^-1 mod 3), B = 3 (3^-1 mod M): then
// W_L^(n k) = W_3^(n1 k1) W_M^(n2 k2).
template <int M, int DIR, typename C> struct pfa3 {
    static constexpr int L = 3 * M;
    static constexpr int inv_mod(int a, int m)
    {
        for (int x = 1; x < m; ++x)
            if ((a * x) % m == 1) return x;
        return 1;
    }
    static constexpr int A = M * inv_mod(M % 3, 3);
    static constexpr int B = 3 * inv_mod(3 % M, M);
    static __device__ __forceinline__ void run(C *a);
};
template <int L, int DIR, typename C> struct rdft;
template <int M, int DIR, typename C> __device__ __forceinline__ void pfa3<M, DIR, C>::run(C *a)
{
    C y[3][M];
#pragma unroll
    for (int n2 = 0; n2 < M; ++n2) {
        C t[3];
#pragma unroll
        for (int n1 = 0; n1 < 3; ++n1) t[n1] = a[(M * n1 + 3 * n2) % L];
        rdft<3, DIR, C>::run(t);
#pragma unroll
        for (int k1 = 0; k1 < 3; ++k1) y[k1][n2] = t[k1];
    }
#pragma unroll
    for (int k1 = 0; k1 < 3; ++k1) {
        rdft<M, DIR, C>::run(y[k1]);
#pragma unroll
        for (int k2 = 0; k2 < M; ++k2) a[(A * k1 + B * k2) % L] = y[k1][k2];
    }
}
#define EMIDA_GB_PFA3(LEN, M)                                                              \
    template <int DIR, typename C> struct rdft<LEN, DIR, C> {                              \
        static __device__ __forceinline__ void run(C *a) { pfa3<M, DIR, C>::run(a); }      \
        static __device__ __forceinline__ void run_half(C *a)                              \
        {                                                                                  \
            using T = decltype(C::x);                                                      \
            _Pragma("unroll") for (int n = LEN / 2; n < LEN; ++n) a[n] = cmake<C>((T)0, (T)0); \
            pfa3<M, DIR, C>::run(a);                                                       \
        }                                                                                  \
    };
EMIDA_GB_PFA3(6, 2)
EMIDA_GB_PFA3(12, 4)
EMIDA_GB_PFA3(24, 8)
#undef EMIDA_GB_PFA3

// Length 3: X0 = a0 + s, X1,2 = a0 - s/2 +- DIR i (sqrt(3)/2) d, s = a1 + a2, d = a1 - a2.
template <int DIR, typename C> struct rdft<3, DIR, C> {
    static __device__ __forceinline__ void run(C *a)
    {
        using T = decltype(C::x);
        const T h = (T)0.8660254037844386467637232;  // sqrt(3)/2
        C s = cadd(a[1], a[2]), d = csub(a[1], a[2]);
        C t = cmake<C>(a[0].x - (T)0.5 * s.x, a[0].y - (T)0.5 * s.y);
        // DIR * i * h * d
        C r = cmake<C>(-(T)DIR * h * d.y, (T)DIR * h * d.x);
        a[0] = cadd(a[0], s);
        a[1] = cadd(t, r);
        a[2] = csub(t, r);
    }
};

// One 1-D transform of length N = G * E carried by G consecutive lanes
// (G = 4 or 8), E values per lane; lane t holds element n = t + G*j in
// register j before and after (self-sorting):
//   n = t + G m, k = k1 + E k2:
//   X[k1 + E k2] = sum_t W_G^{t k2} W_N^{t k1} sum_m x[t + G m] W_E^{m k1}.
// Pass 1 is an E-point DFT over m in registers, then the twiddle, then an
// exchange through the group's own line of N slots (shared memory, reached
// through `line`), then pass 2: E/G G-point DFTs over t.  The exchange slot of
// A'[t][k1] is G*k1 + ((t + k1) mod G): the G lanes' writes (fixed k1) and reads
// (fixed t) fall in G different rows or slots.
// tw: this direction's inter-pass twiddles laid out [lane][k1] with the row
// stride tw_stride, tw[t * TS + k1] = W_N^{t*k1}.  FP32 rows hold an even
// number of slots, so that two twiddles arrive in one 16-byte load, and the
// strides keep the G rows a group reads in distinct banks.  mask: the lanes of
// the warp's groups that run this transform together (whole groups; every
// lane named must call it).
template <int N, int G, typename C> constexpr int tw_stride() { return N / G + (sizeof(C) == 8 ? 2 : 1); }

template <int N, int DIR, bool HALF_INPUT, typename T, int G, typename Line>
__device__ __forceinline__ void group_fft(cplx<T> *v, int t, const Line &line,
                                          const cplx<T> *__restrict__ tw,
                                          unsigned mask = 0xffffffffu)
{
    using C = cplx<T>;
    constexpr int E = N / G;
    static_assert(E % G == 0, "pass 2 needs a whole number of G-point DFTs per lane");
    if (HALF_INPUT)
        rdft<E, DIR, C>::run_half(v);
    else
        rdft<E, DIR, C>::run(v);
    constexpr int TS = tw_stride<N, G, C>();
    const C *twt = tw + t * TS;
    if constexpr (sizeof(C) == 8) {
        static_assert(E % 2 == 0, "twiddles come in pairs");
#pragma unroll
        for (int k1 = 0; k1 < E; k1 += 2) {
            const float4 w = *reinterpret_cast<const float4 *>(twt + k1);
            if (k1 > 0) v[k1] = cmul(v[k1], cmake<C>(w.x, w.y));
            v[k1 + 1] = cmul(v[k1 + 1], cmake<C>(w.z, w.w));
        }
    } else {
#pragma unroll
        for (int k1 = 1; k1 < E; ++k1) v[k1] = cmul(v[k1], twt[k1]);
    }
    __syncwarp(mask);
#pragma unroll
    for (int k1 = 0; k1 < E; ++k1) *line(G * k1 + ((t + k1) & (G - 1))) = v[k1];
    __syncwarp(mask);
#pragma unroll
    for (int i = 0; i < E / G; ++i) {
        C a[G];
#pragma unroll
        for (int s = 0; s < G; ++s) a[s] = *line(G * t + G * G * i + ((s + t) & (G - 1)));
        rdft<G, DIR, C>::run(a);
#pragma unroll
        for (int k2 = 0; k2 < G; ++k2) v[i + (E / G) * k2] = a[k2];
    }
    __syncwarp(mask);
}

}  // namespace emida_gb
