// deformation.cu -- the step after the path: per pattern, the projective map
// (the deformation gradient up to scale) that carries the ROI centres to their
// displaced positions, as python/process_offsets.py:83-104 computes it.  The
// 2S x 9 homogeneous system built from the ROI offsets is solved for the unit
// vector minimising |A x|: the right singular vector of the smallest singular
// value, reshaped to 3 x 3 and divided by its [2][2] entry.
//
// FP64, a warp per pattern, or per two patterns where the batch has two
// patterns per SM and both systems fit shared memory.  Each system sits in shared memory column
// by column; a Householder QR reduces it to a 9 x 9 triangle R with the same
// right singular vectors, and a one-sided (Hestenes) Jacobi SVD orthogonalises
// R's nine columns by plane rotations: the accumulated rotations are the right
// singular vectors and the column norms the singular values.  The QR costs
// about a tenth of the FP64 work of running the rotations over all 2S rows.
// Optionally a quality mask drops ROIs whose fitted peak is not a clear
// maximum, as jove/analyze.py:44-56 does (det of the negated quadratic's
// Hessian <= min_det), and a pattern with ten or fewer good ROIs yields NaN.
#include <cmath>

#include "deformation.cuh"

namespace emida_gb {
namespace {

constexpr int NC = 9;          // unknowns
constexpr int MAX_SWEEPS = 40;

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// 16-lane sum: each half-warp reduces its own values
__device__ __forceinline__ double half_sum(double v)
{
#pragma unroll
    for (int o = 8; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Patterns per warp (PPW = 2): the warp builds and QR-reduces each pattern's
// system in turn, then each half-warp runs one pattern's 9 x 9 Jacobi SVD, so
// the FP64 instructions of the rotations (nine active lanes of sixteen) serve
// two patterns at once.  PPW = 1 where two systems do not fit shared memory:
// both halves then run the same pattern's SVD and the lower one writes it.
template <int PPW>
__global__ void __launch_bounds__(32)
    k_homography(const double *__restrict__ mids, const double *__restrict__ offsets, uint32_t n_rois,
                 uint32_t patterns, double cx, double cy, double cz, const double *__restrict__ coefs,
                 double min_det, double *__restrict__ out)
{
    extern __shared__ double sm[];
    const uint32_t rows = 2 * n_rois;
    const size_t set = (size_t)NC * rows + 2 * NC * NC;  // one pattern's A, V and B
    const int lane = threadIdx.x;
    uint32_t kept0 = 0, kept1 = 0;

#pragma unroll 1
    for (int hp = 0; hp < PPW; ++hp) {
        // a missing last pattern (odd count) runs on a copy of the last and is not written
        const uint32_t pat = min(blockIdx.x * PPW + hp, patterns - 1);
        double *A = sm + hp * set;       // column j: A[j * rows + i]
        double *V = A + NC * rows;       // V[r * NC + c], starts as the identity
        double *B = V + NC * NC;         // R of A = QR, column-major, B[c * NC + r]
        const double *off = offsets + (size_t)pat * n_rois * 2;
        const double *q = coefs ? coefs + (size_t)pat * n_rois * 6 : nullptr;

        // the system of process_offsets.py:85-99, masked rows left at zero
        uint32_t kept = 0;
        for (uint32_t r = lane; r < n_rois; r += 32) {
            bool keep = true;
            if (q) {
                const double a = -q[6 * r + 3], b = -q[6 * r + 4] / 2, c = -q[6 * r + 5];
                keep = a * c - b * b > min_det;
            }
            kept += keep;
            const double a = mids[2 * r] - cx, b = mids[2 * r + 1] - cy, z = cz;
            const double c = a + off[2 * r], d = b + off[2 * r + 1];
            const double e0[NC] = {-a * z, -b * z, -z * z, 0, 0, 0, a * c, b * c, z * c};
            const double e1[NC] = {0, 0, 0, -a * z, -b * z, -z * z, a * d, b * d, z * d};
#pragma unroll
            for (int j = 0; j < NC; ++j) {
                A[j * rows + 2 * r] = keep ? e0[j] : 0.0;
                A[j * rows + 2 * r + 1] = keep ? e1[j] : 0.0;
            }
        }
        for (int i = lane; i < NC * NC; i += 32) V[i] = (i / NC == i % NC) ? 1.0 : 0.0;
#pragma unroll
        for (int o = 16; o; o >>= 1) kept += __shfl_xor_sync(0xffffffffu, kept, o);
        if (hp == 0)
            kept0 = kept;
        else
            kept1 = kept;
        __syncwarp();

        // Householder QR, A = QR: the right singular vectors of A are those of
        // the 9 x 9 triangle R, so the iterative part below works on nine rows only
        for (int k = 0; k < NC; ++k) {
            double *ak = A + k * rows;
            double n2 = 0;
            for (uint32_t i = k + lane; i < rows; i += 32) n2 += ak[i] * ak[i];
            n2 = warp_sum(n2);
            const double x0 = ak[k];
            __syncwarp();
            if (n2 == 0.0) continue;  // the column is zero from row k down: R[k][k] = 0
            const double alpha = x0 >= 0 ? -sqrt(n2) : sqrt(n2);
            const double vtv = 2.0 * (n2 - alpha * x0);  // |x - alpha e_k|^2
            if (lane == 0) ak[k] = x0 - alpha;          // the reflector v, in place
            __syncwarp();
            for (int j = k + 1; j < NC; ++j) {
                double *aj = A + j * rows;
                double w = 0;
                for (uint32_t i = k + lane; i < rows; i += 32) w += ak[i] * aj[i];
                w = warp_sum(w);
                const double f = 2.0 * w / vtv;
                for (uint32_t i = k + lane; i < rows; i += 32) aj[i] -= f * ak[i];
                __syncwarp();
            }
            if (lane == 0) ak[k] = alpha;
            __syncwarp();
        }
        for (int i = lane; i < NC * NC; i += 32) {
            const int c = i / NC, r = i % NC;
            B[i] = r <= c ? A[c * rows + r] : 0.0;
        }
        __syncwarp();
    }

    // cyclic one-sided Jacobi sweeps on each pattern's R: half-warp hp holds
    // pattern hp, its lane r < 9 row r.  Each half rotates by its own tests; a
    // sweep without a rotation in either half ends the iteration.
    const int hp = PPW == 2 ? lane >> 4 : 0, r = lane & 15;
    const bool writer = PPW == 2 || lane < 16;
    double *V = sm + hp * set + NC * rows;
    double *B = V + NC * NC;
    // the columns' squared norms, summed again only when a rotation changed the
    // column (the same sums over the same values: nothing but the work changes)
    double nrm[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        const double x = r < NC ? B[j * NC + r] : 0.0;
        nrm[j] = half_sum(x * x);
    }
    for (int sweep = 0; sweep < MAX_SWEEPS; ++sweep) {
        bool rotated = false;
#pragma unroll
        for (int p = 0; p < NC - 1; ++p) {
#pragma unroll
            for (int k = p + 1; k < NC; ++k) {
                const double x = r < NC ? B[p * NC + r] : 0.0;
                const double y = r < NC ? B[k * NC + r] : 0.0;
                const double al = nrm[p], be = nrm[k], ga = half_sum(x * y);
                // |ga| <= 1e-15 sqrt(al be), squared (NaN columns fail it and rotate)
                const bool rot = !(al == 0.0 || be == 0.0 || ga * ga <= 1e-30 * (al * be));
                if (rot) {
                    rotated = true;
                    // The angle only steers the sweep: t = tan of the Jacobi angle
                    // from zeta in FP32.  zeta = (be - al) / (2 ga) is divided in FP32
                    // where both operands' exponents are within 100 of 0 (their
                    // exponent fields read by integer instructions), else in FP64;
                    // an infinite zeta gives t = 0, an underflowed one t = 1, the
                    // limits of t.  The rotation applied must be orthonormal to FP64
                    // rounding, so c = 1 / sqrt(1 + t^2) is refined from an FP32 seed
                    // by two Newton-Raphson steps for the inverse square root,
                    // c <- c (3 - u c^2) / 2, which double the correct bits each.
                    const double dn = be - al, dd = 2.0 * ga;
                    const int en = (__double2hiint(dn) >> 20) & 0x7ff, ed = (__double2hiint(dd) >> 20) & 0x7ff;
                    float zf;
                    if (en > 1023 - 100 && en < 1023 + 100 && ed > 1023 - 100 && ed < 1023 + 100)
                        zf = (float)dn / (float)dd;
                    else
                        zf = (float)(dn / dd);
                    const float az = fabsf(zf);
                    const float tf = az > 1e18f ? 0.5f / zf : copysignf(1.0f, zf) / (az + sqrtf(1.0f + zf * zf));
                    const double t = (double)tf, u = 1.0 + t * t;
                    double c = (double)rsqrtf((float)u);
                    c = c * (1.5 - 0.5 * u * c * c);
                    c = c * (1.5 - 0.5 * u * c * c);
                    const double s = c * t;
                    if (r < NC && writer) {
                        B[p * NC + r] = c * x - s * y;
                        B[k * NC + r] = s * x + c * y;
                        const double vx = V[r * NC + p], vy = V[r * NC + k];
                        V[r * NC + p] = c * vx - s * vy;
                        V[r * NC + k] = s * vx + c * vy;
                    }
                }
                __syncwarp();
                if (__any_sync(0xffffffffu, rot)) {
                    // both halves take part in the sums; an unrotated half sums its
                    // unchanged columns again
                    const double xn = r < NC ? B[p * NC + r] : 0.0;
                    const double yn = r < NC ? B[k * NC + r] : 0.0;
                    nrm[p] = half_sum(xn * xn);
                    nrm[k] = half_sum(yn * yn);
                }
            }
        }
        if (!__any_sync(0xffffffffu, rotated)) break;
    }

    // the smallest singular value's column of V
    int jmin = 0;
    double smin = INFINITY;
    for (int j = 0; j < NC; ++j) {
        const double x = r < NC ? B[j * NC + r] : 0.0;
        const double n2 = half_sum(x * x);
        if (n2 < smin) {
            smin = n2;
            jmin = j;
        }
    }
    const uint32_t pat = blockIdx.x * PPW + hp;
    if (r < NC && writer && pat < patterns) {
        const uint32_t kept = hp ? kept1 : kept0;
        const bool enough = !coefs || kept > 10;
        const double v = V[r * NC + jmin], v22 = V[8 * NC + jmin];
        out[(size_t)pat * NC + r] = enough ? v / v22 : NAN;
    }
}

}  // namespace

// one pattern's system, V and R
static size_t homography_set_bytes(uint32_t n_rois) { return (size_t)(NC * 2 * n_rois + 2 * NC * NC) * sizeof(double); }
static bool homography_two_per_warp(uint32_t n_rois) { return 2 * homography_set_bytes(n_rois) <= 227 * 1024; }


cudaError_t launch_homography(const double *mids, const double *offsets, uint32_t n_rois,
                              uint32_t patterns, double cx, double cy, double cz, const double *coefs,
                              double min_det, double *out, cudaStream_t st)
{
    if (patterns == 0) return cudaSuccess;
    // two patterns per warp once they leave no SM without a warp (at 256
    // patterns on 152 SMs one per warp is 3 % faster; at 2048, two are 2.2x)
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const bool two = homography_two_per_warp(n_rois) && patterns >= 2u * (uint32_t)sms;
    const size_t smem = (two ? 2 : 1) * homography_set_bytes(n_rois);
    auto k = two ? k_homography<2> : k_homography<1>;
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const uint32_t ppw = two ? 2 : 1;
    k<<<(patterns + ppw - 1) / ppw, 32, smem, st>>>(mids, offsets, n_rois, patterns, cx, cy, cz, coefs, min_det,
                                                    out);
    return cudaGetLastError();
}

}  // namespace emida_gb
