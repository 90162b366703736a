/*
 * emida_oracle.c -- CPU FP64 restatement of emida's ROI cross-correlation path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle).  Only tests/, smoke() and bench.py's
 * CPU-baseline / reference arm may load this library; the product never does.
 *
 * Each function cites the reference file:line whose behaviour it restates.
 * Build with -ffp-contract=off so every FP64 product and sum is rounded
 * separately, exactly as written (the device fit mirrors this order).
 */
#include "emida_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static const double EO_PI = 3.14159265358979323846;

/* ---- src/host_helpers.hpp:29-37 ------------------------------------------ */
void eo_hanning(size_t n, double *out)
{
    for (size_t i = 0; i < n; ++i)
        out[i] = 0.5 * (1 - cos(2 * EO_PI * (double)i / (double)(n - 1)));
}

/* ---- src/sum.cu:109-158 / test/sums_serial.hpp:7-32 --------------------- */
void eo_roi_sums_u16(const uint16_t *pics, uint32_t src_w, uint32_t src_h,
                     const uint32_t *begins, uint32_t n_rois,
                     uint32_t slice_w, uint32_t slice_h, uint32_t batch,
                     uint32_t *sums)
{
    size_t area = (size_t)src_w * src_h;
    for (uint32_t b = 0; b < batch; ++b)
        for (uint32_t r = 0; r < n_rois; ++r) {
            uint32_t acc = 0; /* wraps modulo 2^32 like the reference's uint32 */
            const uint16_t *p = pics + b * area;
            for (uint32_t y = 0; y < slice_h; ++y)
                for (uint32_t x = 0; x < slice_w; ++x)
                    acc += p[(size_t)(begins[2 * r + 1] + y) * src_w + begins[2 * r] + x];
            sums[b * n_rois + r] = acc;
        }
}

void eo_roi_sums_f64(const double *pics, uint32_t src_w, uint32_t src_h,
                     const uint32_t *begins, uint32_t n_rois,
                     uint32_t slice_w, uint32_t slice_h, uint32_t batch,
                     double *sums)
{
    size_t area = (size_t)src_w * src_h;
    for (uint32_t b = 0; b < batch; ++b)
        for (uint32_t r = 0; r < n_rois; ++r) {
            double acc = 0;
            const double *p = pics + b * area;
            for (uint32_t y = 0; y < slice_h; ++y)
                for (uint32_t x = 0; x < slice_w; ++x)
                    acc += p[(size_t)(begins[2 * r + 1] + y) * src_w + begins[2 * r] + x];
            sums[b * n_rois + r] = acc;
        }
}

/* ---- src/prepare_pics.cu:11-42 ------------------------------------------- */
void eo_prepare_f64(const void *pics, int32_t in_type, uint32_t src_w, uint32_t src_h,
                    const uint32_t *begins, uint32_t n_rois, uint32_t slice_w,
                    uint32_t slice_h, uint32_t out_w, uint32_t out_h, uint32_t batch,
                    const double *sums_f64, const double *hx, const double *hy,
                    double *out)
{
    size_t area = (size_t)src_w * src_h;
    uint32_t slice_area = slice_w * slice_h;
    for (uint32_t b = 0; b < batch; ++b)
        for (uint32_t r = 0; r < n_rois; ++r) {
            size_t roi = (size_t)b * n_rois + r;
            double mean = sums_f64[roi] / (double)slice_area;
            double *o = out + roi * out_w * out_h;
            for (uint32_t y = 0; y < slice_h; ++y)
                for (uint32_t x = 0; x < slice_w; ++x) {
                    size_t at = b * area + (size_t)(begins[2 * r + 1] + y) * src_w +
                                begins[2 * r] + x;
                    double pix = in_type == EO_IN_U16 ? (double)((const uint16_t *)pics)[at]
                                                      : ((const double *)pics)[at];
                    pix -= mean;
                    pix = pix * hx[x] * hy[y];
                    o[(size_t)y * out_w + x] = pix;
                }
        }
}

void eo_prepare_f32(const uint16_t *pics, uint32_t src_w, uint32_t src_h,
                    const uint32_t *begins, uint32_t n_rois, uint32_t slice_w,
                    uint32_t slice_h, uint32_t out_w, uint32_t out_h, uint32_t batch,
                    const uint32_t *sums, const float *hx, const float *hy, float *out)
{
    size_t area = (size_t)src_w * src_h;
    uint32_t slice_area = slice_w * slice_h;
    for (uint32_t b = 0; b < batch; ++b)
        for (uint32_t r = 0; r < n_rois; ++r) {
            size_t roi = (size_t)b * n_rois + r;
            float mean = (float)sums[roi] / (float)slice_area;
            float *o = out + roi * out_w * out_h;
            for (uint32_t y = 0; y < slice_h; ++y)
                for (uint32_t x = 0; x < slice_w; ++x) {
                    size_t at = b * area + (size_t)(begins[2 * r + 1] + y) * src_w +
                                begins[2 * r] + x;
                    float pix = (float)pics[at];
                    pix -= mean;
                    pix = pix * hx[x] * hy[y];
                    o[(size_t)y * out_w + x] = pix;
                }
        }
}

/* ---- src/cross_corr.cu:11-66 (same loop bounds and order) ---------------- */
void eo_cross_corr_brute(const double *pics, const double *ref, double *res,
                         uint32_t w, uint32_t h, uint32_t res_w, uint32_t res_h,
                         uint32_t ref_slices, uint32_t batch)
{
    int rx = (int)(res_w - 1) / 2, ry = (int)(res_h - 1) / 2;
    size_t n = (size_t)ref_slices * batch;
    for (size_t i = 0; i < n; ++i) {
        const double *p = pics + i * w * h;
        const double *r = ref + (i % ref_slices) * w * h;
        double *o = res + i * res_w * res_h;
        for (uint32_t py = 0; py < res_h; ++py)
            for (uint32_t px = 0; px < res_w; ++px) {
                int sx = (int)px - rx, sy = (int)py - ry;
                int x_beg = sx < 0 ? -sx : 0, y_beg = sy < 0 ? -sy : 0;
                int x_end = (int)w - sx < (int)w ? (int)w - sx : (int)w;
                int y_end = (int)h - sy < (int)h ? (int)h - sy : (int)h;
                double sum = 0;
                for (int y = y_beg; y < y_end; ++y)
                    for (int x = x_beg; x < x_end; ++x)
                        sum += p[(size_t)(y + sy) * w + (x + sx)] * r[(size_t)y * w + x];
                o[(size_t)py * res_w + px] = sum;
            }
    }
}

/* ---- complex FFT (stands in for cuFFT's R2C/C2R, src/cufft_helpers.hpp) -- */
static uint32_t smallest_factor(uint32_t n)
{
    if (n % 4 == 0) return 4;
    if (n % 2 == 0) return 2;
    for (uint32_t p = 3; p * p <= n; p += 2)
        if (n % p == 0) return p;
    return n;
}

/* exp(sign * 2*pi*i * k / n) with k reduced modulo n first. */
static void twiddle(uint64_t k, uint32_t n, int sign, double *c, double *s)
{
    double ang = 2 * EO_PI * (double)(k % n) / (double)n;
    *c = cos(ang);
    *s = sign * sin(ang);
}

/* Decimation in time: x has element stride xs, X is contiguous. */
static void fft_rec(const double *x, size_t xs, double *X, uint32_t n, int sign, double *tmp)
{
    if (n == 1) {
        X[0] = x[0];
        X[1] = x[1];
        return;
    }
    uint32_t p = smallest_factor(n);
    if (p == n) { /* prime length: direct DFT */
        for (uint32_t k = 0; k < n; ++k) {
            double re = 0, im = 0;
            for (uint32_t t = 0; t < n; ++t) {
                double c, s;
                twiddle((uint64_t)t * k, n, sign, &c, &s);
                double a = x[2 * t * xs], b = x[2 * t * xs + 1];
                re += a * c - b * s;
                im += a * s + b * c;
            }
            X[2 * k] = re;
            X[2 * k + 1] = im;
        }
        return;
    }
    uint32_t m = n / p;
    /* sub-transforms into tmp[j*m ...], scratch for their children after that */
    for (uint32_t j = 0; j < p; ++j)
        fft_rec(x + 2 * j * xs, xs * p, tmp + 2 * (size_t)j * m, m, sign, tmp + 2 * (size_t)n);
    for (uint32_t k = 0; k < n; ++k) {
        double re = 0, im = 0;
        for (uint32_t j = 0; j < p; ++j) {
            double c, s;
            twiddle((uint64_t)j * k, n, sign, &c, &s);
            const double *y = tmp + 2 * ((size_t)j * m + k % m);
            re += y[0] * c - y[1] * s;
            im += y[0] * s + y[1] * c;
        }
        X[2 * k] = re;
        X[2 * k + 1] = im;
    }
}

/* Iterative radix-2 decimation in time for power-of-two n, twiddles computed
 * with cos/sin per length and cached per thread. */
static _Thread_local double *tw_cache = NULL;
static _Thread_local uint32_t tw_n = 0;

static void fft_pow2(double *a, uint32_t n, int sign)
{
    if (tw_n != n) {
        free(tw_cache);
        tw_cache = (double *)malloc(sizeof(double) * n);
        for (uint32_t k = 0; k < n / 2; ++k) {
            tw_cache[2 * k] = cos(2 * EO_PI * (double)k / (double)n);
            tw_cache[2 * k + 1] = sin(2 * EO_PI * (double)k / (double)n);
        }
        tw_n = n;
    }
    for (uint32_t i = 1, j = 0; i < n; ++i) {
        uint32_t bit = n >> 1;
        for (; j & bit; bit >>= 1) j ^= bit;
        j ^= bit;
        if (i < j) {
            double t0 = a[2 * i], t1 = a[2 * i + 1];
            a[2 * i] = a[2 * j];
            a[2 * i + 1] = a[2 * j + 1];
            a[2 * j] = t0;
            a[2 * j + 1] = t1;
        }
    }
    for (uint32_t len = 2; len <= n; len <<= 1) {
        const uint32_t half = len / 2, step = n / len;
        for (uint32_t i = 0; i < n; i += len)
            for (uint32_t k = 0; k < half; ++k) {
                const double c = tw_cache[2 * (k * step)], s = sign * tw_cache[2 * (k * step) + 1];
                double *u = a + 2 * (i + k), *v = a + 2 * (i + k + half);
                const double vr = v[0] * c - v[1] * s, vi = v[0] * s + v[1] * c;
                v[0] = u[0] - vr;
                v[1] = u[1] - vi;
                u[0] += vr;
                u[1] += vi;
            }
    }
}

void eo_fft_c2c(double *data, uint32_t n, int inverse)
{
    if (n >= 2 && (n & (n - 1)) == 0) {
        fft_pow2(data, n, inverse ? 1 : -1);
        return;
    }
    /* scratch: each recursion level needs n complex values; depth <= log2(n)+1 */
    size_t levels = 1;
    for (uint32_t t = n; t > 1; t /= 2) ++levels;
    double *tmp = (double *)malloc(sizeof(double) * 2 * (size_t)n * (levels + 1));
    double *out = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    fft_rec(data, 1, out, n, inverse ? 1 : -1, tmp);
    memcpy(data, out, sizeof(double) * 2 * (size_t)n);
    free(out);
    free(tmp);
}

static void fft2d(double *c, uint32_t w, uint32_t h, int inverse)
{
    double *col = (double *)malloc(sizeof(double) * 2 * h);
    for (uint32_t y = 0; y < h; ++y)
        eo_fft_c2c(c + 2 * (size_t)y * w, w, inverse);
    for (uint32_t x = 0; x < w; ++x) {
        for (uint32_t y = 0; y < h; ++y) {
            col[2 * y] = c[2 * ((size_t)y * w + x)];
            col[2 * y + 1] = c[2 * ((size_t)y * w + x) + 1];
        }
        eo_fft_c2c(col, h, inverse);
        for (uint32_t y = 0; y < h; ++y) {
            c[2 * ((size_t)y * w + x)] = col[2 * y];
            c[2 * ((size_t)y * w + x) + 1] = col[2 * y + 1];
        }
    }
    free(col);
}

static double *real_spectrum(const double *real, uint32_t w, uint32_t h)
{
    size_t n = (size_t)w * h;
    double *c = (double *)malloc(sizeof(double) * 2 * n);
    for (size_t i = 0; i < n; ++i) {
        c[2 * i] = real[i];
        c[2 * i + 1] = 0;
    }
    fft2d(c, w, h, 0);
    return c;
}

/* Conjugate product (src/hadamard.cu:39-40) and unnormalised inverse. */
static void corr_from_spectra(double *P, const double *R, uint32_t w2, uint32_t h2, double *out)
{
    size_t n = (size_t)w2 * h2;
    for (size_t i = 0; i < n; ++i) {
        double px = P[2 * i], py = P[2 * i + 1], rx = R[2 * i], ry = R[2 * i + 1];
        P[2 * i] = px * rx + py * ry;
        P[2 * i + 1] = -px * ry + py * rx;
    }
    fft2d(P, w2, h2, 1);
    for (size_t i = 0; i < n; ++i) out[i] = P[2 * i];
}

void eo_cross_corr_fft(const double *pic, const double *ref, uint32_t w2, uint32_t h2,
                       double *out)
{
    double *P = real_spectrum(pic, w2, h2);
    double *R = real_spectrum(ref, w2, h2);
    corr_from_spectra(P, R, w2, h2, out);
    free(P);
    free(R);
}

/* ---- src/maxarg.cu:118-187 (first maximum in row-major order) ----------- */
void eo_maxarg(const double *maps, uint32_t map_size, uint32_t n, uint32_t *idx, double *val)
{
    for (uint32_t i = 0; i < n; ++i) {
        const double *m = maps + (size_t)i * map_size;
        uint32_t best = 0;
        for (uint32_t j = 1; j < map_size; ++j)
            if (m[j] > m[best]) best = j;
        idx[i] = best;
        if (val) val[i] = m[best];
    }
}

/* ---- src/kernels.cuh:22-53 ------------------------------------------------ */
void eo_shift_pos(uint32_t index, int32_t policy, uint32_t cross_w, uint32_t cross_h,
                  uint32_t *px, uint32_t *py)
{
    if (policy == EO_POLICY_BRUTE) {
        *px = index % cross_w;
        *py = index / cross_w;
    } else {
        uint32_t iw = cross_w + 1, ih = cross_h + 1;
        *px = (index % iw + (iw - 1) / 2) % iw;
        *py = (index / iw + (ih - 1) / 2) % ih;
    }
}

static size_t policy_index(int32_t policy, size_t map, uint32_t x, uint32_t y,
                           uint32_t cross_w, uint32_t cross_h)
{
    if (policy == EO_POLICY_BRUTE)
        return map * cross_w * cross_h + (size_t)y * cross_w + x;
    uint32_t iw = cross_w + 1, ih = cross_h + 1;
    uint32_t ix = (x + (iw / 2 + 1)) % iw, iy = (y + (ih / 2 + 1)) % ih;
    return map * iw * ih + (size_t)iy * iw + ix;
}

/* ---- src/extract_neighbors.cu:12-41 -------------------------------------- */
void eo_extract_neighbors(const double *maps, const uint32_t *idx, uint32_t n,
                          int32_t policy, uint32_t cross_w, uint32_t cross_h, int s,
                          double *neigh)
{
    int r = (s - 1) / 2;
    size_t map_size = policy == EO_POLICY_BRUTE ? (size_t)cross_w * cross_h
                                                : (size_t)(cross_w + 1) * (cross_h + 1);
    size_t total = map_size * n;
    for (uint32_t k = 0; k < n; ++k) {
        uint32_t mx, my;
        eo_shift_pos(idx[k], policy, cross_w, cross_h, &mx, &my);
        for (int i = 0; i < s; ++i)
            for (int j = 0; j < s; ++j) {
                int fx = (int)mx - r + i, fy = (int)my - r + j;
                uint32_t cx = fx < 0 ? 0u : (uint32_t)fx;
                if (cx > cross_w) cx = cross_w;
                uint32_t cy = fy < 0 ? 0u : (uint32_t)fy;
                if (cy > cross_h) cy = cross_h;
                size_t at = policy_index(policy, k, cx, cy, cross_w, cross_h);
                neigh[(size_t)k * s * s + (size_t)j * s + i] = at < total ? maps[at] : 0.0;
            }
    }
}

/* ---- exact least-squares matrix (src/subpixel_max.cpp:22-58, A_gen.py) --- */
typedef __int128 i128;
typedef struct { i128 n, d; } frac;

static i128 gcd128(i128 a, i128 b)
{
    if (a < 0) a = -a;
    if (b < 0) b = -b;
    while (b) {
        i128 t = a % b;
        a = b;
        b = t;
    }
    return a;
}
static frac fr(i128 n, i128 d)
{
    if (d < 0) {
        n = -n;
        d = -d;
    }
    i128 g = gcd128(n, d);
    if (g > 1) {
        n /= g;
        d /= g;
    }
    frac f = {n, d};
    return f;
}
static frac fadd(frac a, frac b) { return fr(a.n * b.d + b.n * a.d, a.d * b.d); }
static frac fsub(frac a, frac b) { return fr(a.n * b.d - b.n * a.d, a.d * b.d); }
static frac fmul(frac a, frac b)
{
    frac x = fr(a.n, b.d), y = fr(b.n, a.d); /* cross-reduce first */
    return fr(x.n * y.n, x.d * y.d);
}
static frac fdiv(frac a, frac b) { return fmul(a, fr(b.d, b.n)); }

int eo_lstsq_matrix(int s, double *out)
{
    if (s != 3 && s != 5 && s != 7 && s != 9) return -1;
    int np = s * s;
    /* A[k][c] for point k = y*s + x: (1, x, y, x^2, xy, y^2) */
    i128 A[81][6];
    for (int y = 0; y < s; ++y)
        for (int x = 0; x < s; ++x) {
            int k = y * s + x;
            A[k][0] = 1;
            A[k][1] = x;
            A[k][2] = y;
            A[k][3] = x * x;
            A[k][4] = x * y;
            A[k][5] = y * y;
        }
    /* augmented [A^T A | A^T], Gauss-Jordan in exact rationals */
    frac M[6][6 + 81];
    for (int i = 0; i < 6; ++i) {
        for (int j = 0; j < 6; ++j) {
            i128 acc = 0;
            for (int k = 0; k < np; ++k) acc += A[k][i] * A[k][j];
            M[i][j] = fr(acc, 1);
        }
        for (int k = 0; k < np; ++k) M[i][6 + k] = fr(A[k][i], 1);
    }
    int cols = 6 + np;
    for (int c = 0; c < 6; ++c) {
        int piv = c;
        while (piv < 6 && M[piv][c].n == 0) ++piv;
        if (piv == 6) return -1;
        if (piv != c)
            for (int j = 0; j < cols; ++j) {
                frac t = M[c][j];
                M[c][j] = M[piv][j];
                M[piv][j] = t;
            }
        frac p = M[c][c];
        for (int j = 0; j < cols; ++j) M[c][j] = fdiv(M[c][j], p);
        for (int i = 0; i < 6; ++i) {
            if (i == c || M[i][c].n == 0) continue;
            frac f = M[i][c];
            for (int j = 0; j < cols; ++j) M[i][j] = fsub(M[i][j], fmul(f, M[c][j]));
        }
    }
    for (int i = 0; i < 6; ++i)
        for (int k = 0; k < np; ++k)
            out[i * np + k] = (double)M[i][6 + k].n / (double)M[i][6 + k].d;
    (void)fadd;
    return 0;
}

/* ---- src/subpixel_max.hpp:14-29, :42-67, :76-97 --------------------------- */
int eo_subpixel_max(const double *neigh, int s, uint32_t n, double *sub, double *coefs)
{
    double mat[6 * 81];
    if (eo_lstsq_matrix(s, mat) != 0) return -1;
    int np = s * s;
    for (uint32_t i = 0; i < n; ++i) {
        const double *v = neigh + (size_t)i * np;
        double c[6];
        for (int j = 0; j < 6; ++j) {
            double acc = 0;
            for (int k = 0; k < np; ++k) acc += mat[j * np + k] * v[k];
            c[j] = acc;
        }
        double a = c[0], b = c[1], cc = c[2], d = c[3], e = c[4], f = c[5];
        double y = (b * e - 2 * cc * d) / (4 * f * d - e * e);
        double x = (-e * y - b) / (2 * d);
        sub[2 * i] = x;
        sub[2 * i + 1] = y;
        if (coefs) {
            coefs[6 * i + 0] = a;
            coefs[6 * i + 1] = b;
            coefs[6 * i + 2] = cc;
            coefs[6 * i + 3] = d;
            coefs[6 * i + 4] = e;
            coefs[6 * i + 5] = f;
        }
    }
    return 0;
}

/* ---- the whole path: src/gpu_offset.hpp:127-301 -------------------------- */
int eo_get_offsets(const eo_params *p, const void *ref_pattern, const void *pics,
                   double *offsets, double *coefs, uint32_t *peaks)
{
    if (p->fitsize != 3 && p->fitsize != 5 && p->fitsize != 7 && p->fitsize != 9) return -1;
    if (p->policy != EO_POLICY_BRUTE && p->policy != EO_POLICY_FFT) return -2;
    if (p->slice_w == 0 || p->slice_h == 0 || p->n_rois == 0 || p->batch == 0) return -3;
    for (uint32_t r = 0; r < p->n_rois; ++r)
        if ((uint64_t)p->begins[2 * r] + p->slice_w > p->src_w ||
            (uint64_t)p->begins[2 * r + 1] + p->slice_h > p->src_h)
            return -4;
    uint32_t sw = p->slice_w, sh = p->slice_h, S = p->n_rois;
    size_t N = (size_t)S * p->batch;
    uint32_t cw, ch, mw, mh, pw, ph;
    if (p->policy == EO_POLICY_FFT) {
        cw = 2 * sw - 1;
        ch = 2 * sh - 1;
        mw = pw = 2 * sw;
        mh = ph = 2 * sh;
    } else {
        cw = p->cross_w;
        ch = p->cross_h;
        if (cw == 0 || ch == 0 || cw > 2 * sw - 1 || ch > 2 * sh - 1) return -5;
        mw = cw;
        mh = ch;
        pw = sw;
        ph = sh;
    }
    double *hx = (double *)malloc(sizeof(double) * sw);
    double *hy = (double *)malloc(sizeof(double) * sh);
    eo_hanning(sw, hx);
    eo_hanning(sh, hy);

    double *ref_sums = (double *)malloc(sizeof(double) * S);
    double *pic_sums = (double *)malloc(sizeof(double) * N);
    if (p->in_type == EO_IN_U16) {
        uint32_t *u = (uint32_t *)malloc(sizeof(uint32_t) * N);
        eo_roi_sums_u16((const uint16_t *)ref_pattern, p->src_w, p->src_h, p->begins, S, sw,
                        sh, 1, u);
        for (uint32_t i = 0; i < S; ++i) ref_sums[i] = (double)u[i];
        eo_roi_sums_u16((const uint16_t *)pics, p->src_w, p->src_h, p->begins, S, sw, sh,
                        p->batch, u);
        for (size_t i = 0; i < N; ++i) pic_sums[i] = (double)u[i];
        free(u);
    } else {
        eo_roi_sums_f64((const double *)ref_pattern, p->src_w, p->src_h, p->begins, S, sw,
                        sh, 1, ref_sums);
        eo_roi_sums_f64((const double *)pics, p->src_w, p->src_h, p->begins, S, sw, sh,
                        p->batch, pic_sums);
    }
    double *refp = (double *)calloc((size_t)S * pw * ph, sizeof(double));
    double *picp = (double *)calloc(N * pw * ph, sizeof(double));
    eo_prepare_f64(ref_pattern, p->in_type, p->src_w, p->src_h, p->begins, S, sw, sh, pw, ph,
                   1, ref_sums, hx, hy, refp);
    eo_prepare_f64(pics, p->in_type, p->src_w, p->src_h, p->begins, S, sw, sh, pw, ph,
                   p->batch, pic_sums, hx, hy, picp);

    size_t msize = (size_t)mw * mh;
    double *maps = (double *)malloc(sizeof(double) * N * msize);
    if (p->policy == EO_POLICY_BRUTE) {
        eo_cross_corr_brute(picp, refp, maps, sw, sh, cw, ch, S, p->batch);
    } else {
        double **R = (double **)malloc(sizeof(double *) * S);
        for (uint32_t r = 0; r < S; ++r) R[r] = real_spectrum(refp + (size_t)r * msize, pw, ph);
        for (size_t i = 0; i < N; ++i) {
            double *P = real_spectrum(picp + i * msize, pw, ph);
            corr_from_spectra(P, R[i % S], pw, ph, maps + i * msize);
            free(P);
        }
        for (uint32_t r = 0; r < S; ++r) free(R[r]);
        free(R);
    }
    uint32_t *idx = (uint32_t *)malloc(sizeof(uint32_t) * N);
    eo_maxarg(maps, (uint32_t)msize, (uint32_t)N, idx, NULL);
    int s = p->fitsize, rr = (s - 1) / 2;
    double *neigh = (double *)malloc(sizeof(double) * N * s * s);
    eo_extract_neighbors(maps, idx, (uint32_t)N, p->policy, cw, ch, s, neigh);
    double *sub = (double *)malloc(sizeof(double) * 2 * N);
    eo_subpixel_max(neigh, s, (uint32_t)N, sub, coefs);
    for (size_t i = 0; i < N; ++i) {
        uint32_t mx, my;
        eo_shift_pos(idx[i], p->policy, cw, ch, &mx, &my);
        offsets[2 * i] = -((int)mx - ((int)cw / 2) - rr + sub[2 * i]);
        offsets[2 * i + 1] = -((int)my - ((int)ch / 2) - rr + sub[2 * i + 1]);
        if (peaks) peaks[i] = idx[i];
    }
    free(sub);
    free(neigh);
    free(idx);
    free(maps);
    free(picp);
    free(refp);
    free(pic_sums);
    free(ref_sums);
    free(hy);
    free(hx);
    return 0;
}
