/*
 * rsf_oracle.c -- CPU restatement of the reference RSF level-set evolution.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: tests/, the
 * smoke() entry and the cpu_baseline / reference arm of bench.py call it as
 * the checker.  No product code path links, loads or calls it.
 *
 * What it restates (paths are relative to the reference project):
 *   CUDA_RSF/main.cpp:152-166   Gaussian taps (p = floor(7 sigma) made odd,
 *                               u = (int)(2 sigma^2), unnormalised)
 *   CUDA_RSF/main.cpp:222-314   per-iteration call order
 *   CUDA_RSF/kernel.cu:248-263  heaviside      H = 0.5(1 + 2/pi atan(phi/eps))
 *   CUDA_RSF/kernel.cu:210-226  multiplication I*H, I*(1-H)
 *   CUDA_RSF/kernel.cu:282-298  inverse        1 - H
 *   CUDA_RSF/kernel.cu:57-125   gradient_dx/dy/dz_cuda (boundary rules below)
 *   CUDA_RSF/kernel.cu:914-933  gradientmagnitude
 *   CUDA_RSF/kernel.cu:173-189  division_grad  g / (|g| + 1e-6), in double
 *   CUDA_RSF/kernel.cu:744-785, 858-909, 228-245  curvature = sum_a D_a(n_a)
 *   CUDA_RSF/kernel.cu:630-684  DIV_cal        "Laplacian" = sum_a D_a(D_a phi)
 *   CUDA_RSF/kernel.cu:1000-1121 separable valid correlation x -> y -> z
 *   CUDA_RSF/kernel.cu:300-362  pad_border     border band := 30
 *   CUDA_RSF/kernel.cu:191-207  division       f = blur(I H) / blur(H)
 *   CUDA_RSF/kernel.cu:25-55    Eout_Ein_calculation (box radius (int)sigma2)
 *   CUDA_RSF/kernel.cu:265-280  deri_heaviside delta = (1/pi) eps/(eps^2+phi^2)
 *   CUDA_RSF/kernel.cu:365-387  Final_phi      explicit update
 *   CUDA_RSF/main.cpp:174-183   phi0 = sdf(seed - 13): this project's own
 *                               definition (tiralib's sdf is not in the
 *                               reference), see oracle_signed_distance
 * and one mode of this project's own with no counterpart in the reference:
 * the expanded Gaussian data term (data_term = 1, gaussian_data_terms).
 *
 * Arithmetic follows the reference kernels operation by operation.  Every
 * a*b+c that nvcc contracts into a fused multiply-add under its default
 * -fmad=true is written as an explicit fmaf().  The spots the reference
 * evaluates in double (heaviside, deri_heaviside, division_grad, the x/z
 * gradients, the e-term weight) have two definitions, selected by
 * oracle_params.arith (see "Pointwise stages" below).  The file must be built
 * with -ffp-contract=off so that the host compiler adds no contraction of its
 * own (gcc contracts by default on aarch64).
 *
 * Deliberate definitions where the reference is undefined or not restatable:
 *   - voxel 0's x-gradient reads element -1 of the buffer in the reference
 *     (kernel.cu:64-73, size_t underflow); here that read returns element 0.
 *   - the reference calls CUDA's single-precision atanf, whose algorithm is
 *     not public; the portable definition uses this file's own atan.
 *
 * The FP64 twin (oracle_evolve_f64) evaluates the same formulas entirely in
 * double; it is used to state the error of the FP32 paths.
 *
 * Pinning: every stage is checked bit for bit against the outputs of the
 * reference's own kernel.cu, compiled unchanged and run on a GB300
 * (tests/test_reference_kernels.py, fixtures tests/golden/reference_kernels_*.npz);
 * only H differs, through the reference's single-precision atan.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RSF_PI 3.14159265358979323846

/* Parameter block shared with the Python side through ctypes. */
typedef struct {
    float sigma;    /* --sigma  (main.cpp:91) */
    float dt;       /* --dt     (main.cpp:93) */
    float mu;       /* --meu    (main.cpp:94) */
    float lambda1;  /* --e      (main.cpp:95), weight of e_out */
    float lambda2;  /* --e      (main.cpp:95), weight of e_in */
    float nu;       /* --v      (main.cpp:96) */
    float eps;      /* hard-coded 0.2 in kernel.cu:258,275 */
    float sigma2;   /* --sigma2 (main.cpp:97), box radius after (int) */
    int32_t boundary;  /* 0: reference x=0 rule (previous row), 1: clamp */
    int32_t mag_form;  /* contraction order of |g|^2, see grad_mag2() */
    int32_t arith;     /* 0 portable float sequences, 1 reference double spots */
    int32_t data_term; /* 0 the reference's (I - f)^2 / box form, 1 expanded Gaussian */
} oracle_params;

static inline size_t idx3(int64_t x, int64_t y, int64_t z, int64_t W, int64_t H) {
    return ((size_t)z * (size_t)H + (size_t)y) * (size_t)W + (size_t)x;
}

/* ------------------------------------------------------------------------ */
/* Gaussian taps, main.cpp:152-166.                                          */
/* exp is evaluated in double and rounded so the taps are identical on every */
/* host; the reference evaluates expf on the host (MSVC).                     */
/* ------------------------------------------------------------------------ */
int oracle_taps(float sigma, float *taps, int cap) {
    if (!(sigma > 0.0f)) return -1;
    unsigned p = (unsigned)(7.0f * sigma);
    if (p % 2u == 0u) p++;
    float miu = (float)(p / 2u);
    int u = (int)(2.0f * sigma * sigma);
    if (u < 1 || (int)p > cap) return -1;
    float s = sqrtf((float)u * (float)RSF_PI);
    for (unsigned xi = 0; xi < p; xi++) {
        float d = (float)(int)xi - miu;
        float a = (-d * d) / (float)u;
        taps[xi] = (1.0f / s) * (float)exp((double)a);
    }
    return (int)p;
}

/* ------------------------------------------------------------------------ */
/* Pointwise stages.                                                          */
/*                                                                            */
/* Two arithmetic definitions are provided (oracle_params.arith):            */
/*   RSF_ARITH_PORTABLE (0): float-only sequences of correctly rounded IEEE   */
/*     operations (+ - * / sqrt fma).  The reference's double-precision spots */
/*     are evaluated with compensated (double-float) arithmetic, and atan is  */
/*     this file's own polynomial.  Every step is a basic IEEE operation, so  */
/*     any conforming CPU or GPU that performs the same sequence produces the */
/*     same bits.  This is the definition the CUDA path reproduces exactly.   */
/*   RSF_ARITH_REFERENCE (1): the reference's double-precision evaluation     */
/*     with the host libm atan; used to measure how far the portable          */
/*     definition is from the reference's own arithmetic (at most ~1 ulp per  */
/*     stage).                                                                */
/* ------------------------------------------------------------------------ */

/* atan on [-inf, inf] from the identity atan(x) = pi/2 - atan(1/x) (x > 1)   */
/* and atan(u) = u + u^3 R(u^2) on [0, 1], R a degree-8 polynomial fitted     */
/* for this project (weighted least squares towards minimax relative error).  */
/* Max error against the exact atan: 0.95 ulp on [-1, 1], 1.35 ulp beyond.   */
static const float ATAN_R[9] = {
    -0x1.55553e0000000p-2f,
    0x1.9992160000000p-3f,
    -0x1.2422a20000000p-3f,
    0x1.c0a2c00000000p-4f,
    -0x1.584c200000000p-4f,
    0x1.db15280000000p-5f,
    -0x1.ff5ed60000000p-6f,
    0x1.6636cc0000000p-7f,
    -0x1.d727360000000p-10f};
static const float PIO2_HI = 0x1.921fb60000000p+0f;  /* float(pi/2) */
static const float PIO2_LO = -0x1.777a5c0000000p-25f;  /* pi/2 - PIO2_HI */

float oracle_atan(float x) {
    float a = fabsf(x);
    int big = a > 1.0f;
    float u = big ? 1.0f / a : a;
    float z = u * u;
    float r = ATAN_R[8];
    for (int i = 7; i >= 0; i--) r = fmaf(r, z, ATAN_R[i]);
    float t = u * z;
    float p = fmaf(t, r, u);
    float res = big ? (PIO2_HI - p) + PIO2_LO : p;
    return copysignf(res, x);
}

/* 2/pi, 1/pi and 1e-6 as unevaluated float pairs hi + lo (lo = value - hi */
/* rounded to float), written as exact hexadecimal float literals.         */
static const float TWO_PI_HI = 0x1.45f3060000000p-1f;
static const float TWO_PI_LO = 0x1.b939100000000p-26f;
static const float INV_PI_HI = 0x1.45f3060000000p-2f;
static const float INV_PI_LO = 0x1.b939100000000p-27f;
static const float EPS6_HI = 0x1.0c6f7a0000000p-20f;
static const float EPS6_LO = 0x1.6bdb1a0000000p-49f;

/* kernel.cu:258-259: H = 0.5 (1 + (2/pi) atan(phi/eps)); the reference forms */
/* 1 + (2/pi) a in double.  Portable: product and sum kept as exact float    */
/* pairs (Dekker product via fma, Fast2Sum since |(2/pi) a| <= 1).            */
static inline float heaviside_f32(float phi, float eps, int arith) {
    if (arith == 1) {
        float a = (float)atan((double)(phi / eps));
        return (float)(0.5 * fma(2.0 / RSF_PI, (double)a, 1.0));
    }
    float a = oracle_atan(phi / eps);
    float p = TWO_PI_HI * a;
    float pe = fmaf(TWO_PI_HI, a, -p);
    float s = 1.0f + p;
    float se = (1.0f - s) + p;
    float lo = fmaf(TWO_PI_LO, a, pe) + se;
    return 0.5f * (s + lo);
}

/* kernel.cu:275-276: eps*eps + phi*phi contracts to fma(phi, phi, eps*eps);  */
/* the quotient is float and the 1/pi factor is applied in double.            */
static inline float dirac_f32(float phi, float eps, int arith) {
    float q = eps / fmaf(phi, phi, eps * eps);
    if (arith == 1) return (float)((1.0 / RSF_PI) * (double)q);
    float p = INV_PI_HI * q;
    float e = fmaf(INV_PI_HI, q, -p);
    return p + fmaf(INV_PI_LO, q, e);
}

/* kernel.cu:928: sqrt(gx*gx + gy*gy + gz*gz) with nvcc's contraction. */
static inline float grad_mag2(float gx, float gy, float gz, int form) {
    float inner = form == 0 ? fmaf(gx, gx, gy * gy) : fmaf(gy, gy, gx * gx);
    return fmaf(gz, gz, inner);
}

/* kernel.cu:185: n = g / (|g| + 1e-6) with the sum and quotient in double.   */
/* Portable: s + dlo = |g| + 1e-6 by TwoSum, then one Newton correction of    */
/* the quotient g * (1/s) against the pair.                                   */
typedef struct { float s, dlo, rinv; } norm_den;

static inline norm_den norm_den_make(float mag) {
    norm_den d;
    d.s = mag + EPS6_HI;
    float bb = d.s - mag;
    float err = (mag - (d.s - bb)) + (EPS6_HI - bb);
    d.dlo = err + EPS6_LO;
    d.rinv = 1.0f / d.s;
    return d;
}

static inline float normalise_f32(float g, float mag, const norm_den *d, int arith) {
    if (arith == 1) return (float)((double)g / ((double)mag + 1e-6));
    float q0 = g * d->rinv;
    float r = fmaf(-q0, d->s, g);
    r = fmaf(-q0, d->dlo, r);
    return fmaf(r, d->rinv, q0);
}

/* kernel.cu:73-78 and 119-124 evaluate in double; kernel.cu:102 in float. */
static inline float half_diff_d(float r, float l) { return (float)(((double)r - (double)l) / 2.0); }
static inline float half_diff_f(float r, float l) { return (r - l) / 2.0f; }

/* ------------------------------------------------------------------------ */
/* Central differences with the reference's boundary rules.                   */
/*   x: x=W-1 -> (f[W-1]-f[W-2])/2; x=0 -> (f[1] - f[lin-1])/2 (reference)   */
/*      or (f[1]-f[0])/2 (clamp).  kernel.cu:57-79                            */
/*   y: y=0 -> (f[1]-f[0])/2; y=H-1 -> (f[H-1]-f[H-2])/2.  kernel.cu:82-107  */
/*   z: z=0 -> (f[1]-f[0])/2; z=L-1 -> (f[L-1]-f[L-2])/2.  kernel.cu:109-125 */
/* ------------------------------------------------------------------------ */
static void diff_x(const float *f, float *out, int64_t W, int64_t H, int64_t L, int boundary) {
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < L; z++)
        for (int64_t y = 0; y < H; y++)
            for (int64_t x = 0; x < W; x++) {
                size_t i = idx3(x, y, z, W, H);
                size_t ir = (x + 1 < W) ? i + 1 : i;
                size_t il;
                if (x > 0) il = i - 1;
                else if (boundary == 0) il = (i > 0) ? i - 1 : 0;  /* previous linear element */
                else il = i;
                if (x == W - 1 && W > 1) il = i - 1;
                out[i] = half_diff_d(f[ir], f[il]);
            }
}

static void diff_y(const float *f, float *out, int64_t W, int64_t H, int64_t L) {
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < L; z++)
        for (int64_t y = 0; y < H; y++) {
            int64_t yl = y - 1, yr = y + 1;
            if (yl < 0) { yl = 0; yr = 1; }
            else if (yr >= H) { yr = H - 1; yl = yr - 1; }
            for (int64_t x = 0; x < W; x++)
                out[idx3(x, y, z, W, H)] = half_diff_f(f[idx3(x, yr, z, W, H)], f[idx3(x, yl, z, W, H)]);
        }
}

static void diff_z(const float *f, float *out, int64_t W, int64_t H, int64_t L) {
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < L; z++) {
        int64_t zl = z > 0 ? z - 1 : 0;
        int64_t zr = z < L - 1 ? z + 1 : L - 1;
        for (int64_t y = 0; y < H; y++)
            for (int64_t x = 0; x < W; x++)
                out[idx3(x, y, z, W, H)] = half_diff_d(f[idx3(x, y, zr, W, H)], f[idx3(x, y, zl, W, H)]);
    }
}

/* Public per-stage entry: out{x,y,z} = D_{x,y,z} f. */
void oracle_gradient(const float *f, float *gx, float *gy, float *gz,
                     int64_t W, int64_t H, int64_t L, int boundary) {
    diff_x(f, gx, W, H, L, boundary);
    diff_y(f, gy, W, H, L);
    diff_z(f, gz, W, H, L);
}

/* ------------------------------------------------------------------------ */
/* Separable valid correlation, kernel.cu:1000-1049.                          */
/* out[x] = sum_{t ascending} in[x+t] * g[t], accumulated with fma from 0.    */
/* ------------------------------------------------------------------------ */
static void conv_x(const float *in, float *out, int64_t W, int64_t H, int64_t L,
                   const float *g, int k) {
    int64_t Wo = W - k + 1;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < L; z++)
        for (int64_t y = 0; y < H; y++)
            for (int64_t x = 0; x < Wo; x++) {
                const float *row = in + idx3(x, y, z, W, H);
                float acc = 0.0f;
                for (int t = 0; t < k; t++) acc = fmaf(row[t], g[t], acc);
                out[idx3(x, y, z, Wo, H)] = acc;
            }
}

static void conv_y(const float *in, float *out, int64_t W, int64_t H, int64_t L,
                   const float *g, int k) {
    int64_t Ho = H - k + 1;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < L; z++)
        for (int64_t y = 0; y < Ho; y++)
            for (int64_t x = 0; x < W; x++) {
                float acc = 0.0f;
                for (int t = 0; t < k; t++) acc = fmaf(in[idx3(x, y + t, z, W, H)], g[t], acc);
                out[idx3(x, y, z, W, Ho)] = acc;
            }
}

static void conv_z(const float *in, float *out, int64_t W, int64_t H, int64_t L,
                   const float *g, int k) {
    int64_t Lo = L - k + 1;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < Lo; z++)
        for (int64_t y = 0; y < H; y++)
            for (int64_t x = 0; x < W; x++) {
                float acc = 0.0f;
                for (int t = 0; t < k; t++) acc = fmaf(in[idx3(x, y, z + t, W, H)], g[t], acc);
                out[idx3(x, y, z, W, H)] = acc;
            }
}

/*
 * adddevice_convolution_seperable (kernel.cu:1051-1121) followed by
 * pad_border_cal (kernel.cu:300-362): blur `in` with the valid separable
 * correlation and embed the result at offset r = (k-1)/2 of a W x H x L
 * volume whose border band holds 30.  Returns 0, or -1 on allocation failure.
 */
int oracle_blur_padded(const float *in, float *out, int64_t W, int64_t H, int64_t L,
                       const float *g, int k) {
    int64_t r = (k - 1) / 2;
    int64_t Wo = W - k + 1, Ho = H - k + 1, Lo = L - k + 1;
    if (Wo <= 0 || Ho <= 0 || Lo <= 0) {
        size_t n = (size_t)W * H * L;
        for (size_t i = 0; i < n; i++) out[i] = 30.0f;
        return 0;
    }
    float *bx = (float *)malloc(sizeof(float) * (size_t)Wo * H * L);
    float *by = (float *)malloc(sizeof(float) * (size_t)Wo * Ho * L);
    float *bz = (float *)malloc(sizeof(float) * (size_t)Wo * Ho * Lo);
    if (!bx || !by || !bz) { free(bx); free(by); free(bz); return -1; }
    conv_x(in, bx, W, H, L, g, k);
    conv_y(bx, by, Wo, H, L, g, k);
    conv_z(by, bz, Wo, Ho, L, g, k);
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < L; z++)
        for (int64_t y = 0; y < H; y++)
            for (int64_t x = 0; x < W; x++) {
                int border = x < r || x >= Wo + r || y < r || y >= Ho + r || z < r || z >= Lo + r;
                out[idx3(x, y, z, W, H)] = border ? 30.0f
                    : bz[idx3(x - r, y - r, z - r, Wo, Ho)];
            }
    free(bx); free(by); free(bz);
    return 0;
}

/*
 * Eout_Ein_calculation, kernel.cu:25-55.  s = (int)sigma2.  The weight is
 * 1/(2s+1)^2 in double; the float accumulator is widened, fused with the
 * double product and rounded back on every term, as the reference does.
 * Neighbours outside the volume are skipped.  Loop order: y, x, z.
 */
static void data_terms(const float *I, const float *fo, const float *fi, float *eo, float *ei,
                       int64_t W, int64_t H, int64_t L, int s) {
    double w = 1.0 / pow((double)(2 * s + 1), 2.0);
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < L; z++)
        for (int64_t y = 0; y < H; y++)
            for (int64_t x = 0; x < W; x++) {
                size_t c = idx3(x, y, z, W, H);
                float s1 = 0.0f, s2 = 0.0f;
                for (int u = -s; u <= s; u++)
                    for (int v = -s; v <= s; v++)
                        for (int q = -s; q <= s; q++) {
                            int64_t yy = y + u, xx = x + v, zz = z + q;
                            if (yy < 0 || yy >= H || xx < 0 || xx >= W || zz < 0 || zz >= L) continue;
                            float In = I[idx3(xx, yy, zz, W, H)];
                            float d1 = In - fo[c], d2 = In - fi[c];
                            s1 = (float)fma(w * (double)d1, (double)d1, (double)s1);
                            s2 = (float)fma(w * (double)d2, (double)d2, (double)s2);
                        }
                eo[c] = s1;
                ei[c] = s2;
            }
}

/*
 * The expanded Gaussian data term (data_term = 1; no counterpart in the
 * reference, whose kernel.cu:25-55 takes (I - f)^2 at the voxel).  It is the
 * region-scalable fitting energy's data term written out:
 *   e_i(c) = I(c)^2 (K*1)(c) - 2 I(c) (K*f_i)(c) + (K*f_i^2)(c)
 * on the valid region of the blur, where K is the same valid separable
 * correlation as the local fits (x, then y, then z, taps ascending, fused
 * multiply-adds from +0) and f_i the full-volume fit field (1 in the border
 * band).  K*1 is the same constant s3 at every valid voxel.  FP32 sequence:
 *   b = fmaf(I*I, s3, K*f^2);  e = fmaf(-2*I, K*f, b).
 * The border band keeps the reference form (I - 1)^2.
 */
static float ones_correlation(const float *g, int k) {
    float sx = 0.0f, sy = 0.0f, s3 = 0.0f;
    for (int t = 0; t < k; t++) sx = fmaf(1.0f, g[t], sx);
    for (int t = 0; t < k; t++) sy = fmaf(sx, g[t], sy);
    for (int t = 0; t < k; t++) s3 = fmaf(sy, g[t], s3);
    return s3;
}

static int gaussian_data_terms(const float *I, const float *fo, const float *fi, float *eo, float *ei,
                               int64_t W, int64_t H, int64_t L, const float *g, int k) {
    data_terms(I, fo, fi, eo, ei, W, H, L, 0);  /* the border band's form everywhere first */
    int64_t r = (k - 1) / 2, Wo = W - k + 1, Ho = H - k + 1, Lo = L - k + 1;
    if (Wo <= 0 || Ho <= 0 || Lo <= 0) return 0;
    size_t n = (size_t)W * H * L, nv = (size_t)Wo * Ho * Lo;
    float *fld = (float *)malloc(sizeof(float) * n);
    float *bx = (float *)malloc(sizeof(float) * (size_t)Wo * H * L);
    float *by = (float *)malloc(sizeof(float) * (size_t)Wo * Ho * L);
    float *kb = (float *)malloc(sizeof(float) * nv * 4);
    if (!fld || !bx || !by || !kb) { free(fld); free(bx); free(by); free(kb); return -1; }
    const float *src[2] = {fo, fi};
    for (int j = 0; j < 4; j++) {
        const float *f = src[j >> 1];
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < (int64_t)n; i++) fld[i] = (j & 1) ? f[i] * f[i] : f[i];
        conv_x(fld, bx, W, H, L, g, k);
        conv_y(bx, by, Wo, H, L, g, k);
        conv_z(by, kb + (size_t)j * nv, Wo, Ho, L, g, k);
    }
    const float s3 = ones_correlation(g, k);
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < Lo; z++)
        for (int64_t y = 0; y < Ho; y++)
            for (int64_t x = 0; x < Wo; x++) {
                size_t v = idx3(x, y, z, Wo, Ho), c = idx3(x + r, y + r, z + r, W, H);
                float Ic = I[c], a = Ic * Ic, m2 = -2.0f * Ic;
                eo[c] = fmaf(m2, kb[v], fmaf(a, s3, kb[nv + v]));
                ei[c] = fmaf(m2, kb[2 * nv + v], fmaf(a, s3, kb[3 * nv + v]));
            }
    free(fld); free(bx); free(by); free(kb);
    return 0;
}

/*
 * Final_phi, kernel.cu:384, with nvcc's contraction:
 *   phi - (dh*(e*(Eo-Ei)))*dt + ((v*dt)*dh)*nd + meu*(dt*(div-nd))
 *   = fma(meu, dt*(div-nd), fma((v*dt)*dh, nd, fma(-(dh*(e*(Eo-Ei))), dt, phi)))
 * With lambda1 != lambda2 the data factor is lambda1*Eo - lambda2*Ei.
 */
static inline float update_f32(float phi, float dh, float eo, float ei, float kap, float lap,
                               const oracle_params *p) {
    float data = (p->lambda1 == p->lambda2) ? p->lambda1 * (eo - ei)
                                            : (p->lambda1 * eo) - (p->lambda2 * ei);
    float a = fmaf(-(dh * data), p->dt, phi);
    float b = fmaf((p->nu * p->dt) * dh, kap, a);
    return fmaf(p->mu, p->dt * (lap - kap), b);
}

/* ------------------------------------------------------------------------ */
/* One iteration, main.cpp:233-300.  Optional `dbg` receives 8 N-sized       */
/* fields in order: f_out, f_in, e_out, e_in, delta, kappa, lap, |grad|.      */
/* ------------------------------------------------------------------------ */
int oracle_step_f32(const float *phi, const float *I, float *phi_out,
                    int64_t W, int64_t H, int64_t L, const oracle_params *p, float *dbg) {
    float g[512];
    int k = oracle_taps(p->sigma, g, 512);
    if (k < 0) return -2;
    size_t n = (size_t)W * H * L;
    enum { F_HO, F_HI, F_IO, F_II, F_GX, F_GY, F_GZ, F_MAG, F_NX, F_NY, F_NZ,
           F_T0, F_T1, F_T2, F_KAP, F_LAP, F_BIO, F_BHO, F_BII, F_BHI,
           F_FO, F_FI, F_EO, F_EI, F_DH, F_COUNT };
    float *buf = (float *)malloc(sizeof(float) * n * F_COUNT);
    if (!buf) return -1;
    float *F[F_COUNT];
    for (int i = 0; i < F_COUNT; i++) F[i] = buf + (size_t)i * n;

    /* heaviside, multiplication, inverse, multiplication: main.cpp:234-246 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        float h = heaviside_f32(phi[i], p->eps, p->arith);
        F[F_HO][i] = h;
        F[F_IO][i] = I[i] * h;
        float hi = 1.0f - h;
        F[F_HI][i] = hi;
        F[F_II][i] = I[i] * hi;
    }
    /* gradient_cal, gradientmagnitude_cal, division_nDIV: main.cpp:250-254 */
    oracle_gradient(phi, F[F_GX], F[F_GY], F[F_GZ], W, H, L, p->boundary);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        float m = sqrtf(grad_mag2(F[F_GX][i], F[F_GY][i], F[F_GZ][i], p->mag_form));
        norm_den d = norm_den_make(m);
        F[F_MAG][i] = m;
        F[F_NX][i] = normalise_f32(F[F_GX][i], m, &d, p->arith);
        F[F_NY][i] = normalise_f32(F[F_GY][i], m, &d, p->arith);
        F[F_NZ][i] = normalise_f32(F[F_GZ][i], m, &d, p->arith);
    }
    /* gradient_cal_3_input + normalized_div_plus: main.cpp:256-258 */
    diff_x(F[F_NX], F[F_T0], W, H, L, p->boundary);
    diff_y(F[F_NY], F[F_T1], W, H, L);
    diff_z(F[F_NZ], F[F_T2], W, H, L);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) F[F_KAP][i] = F[F_T0][i] + F[F_T1][i] + F[F_T2][i];
    /* DIV_cal: main.cpp:260 */
    diff_x(F[F_GX], F[F_T0], W, H, L, p->boundary);
    diff_y(F[F_GY], F[F_T1], W, H, L);
    diff_z(F[F_GZ], F[F_T2], W, H, L);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) F[F_LAP][i] = F[F_T0][i] + F[F_T1][i] + F[F_T2][i];
    /* blurs, pads, divisions: main.cpp:268-289 */
    int rc = 0;
    rc |= oracle_blur_padded(F[F_IO], F[F_BIO], W, H, L, g, k);
    rc |= oracle_blur_padded(F[F_HO], F[F_BHO], W, H, L, g, k);
    rc |= oracle_blur_padded(F[F_II], F[F_BII], W, H, L, g, k);
    rc |= oracle_blur_padded(F[F_HI], F[F_BHI], W, H, L, g, k);
    if (rc) { free(buf); return -1; }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        F[F_FO][i] = F[F_BIO][i] / F[F_BHO][i];
        F[F_FI][i] = F[F_BII][i] / F[F_BHI][i];
    }
    /* adddevice: main.cpp:293 */
    if (p->data_term == 1) {
        if (gaussian_data_terms(I, F[F_FO], F[F_FI], F[F_EO], F[F_EI], W, H, L, g, k)) { free(buf); return -1; }
    } else {
        data_terms(I, F[F_FO], F[F_FI], F[F_EO], F[F_EI], W, H, L, (int)p->sigma2);
    }
    /* deri_heaviside_cal, Final_PHI_cal: main.cpp:296-300 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        float dh = dirac_f32(phi[i], p->eps, p->arith);
        F[F_DH][i] = dh;
        phi_out[i] = update_f32(phi[i], dh, F[F_EO][i], F[F_EI][i], F[F_KAP][i], F[F_LAP][i], p);
    }
    if (dbg) {
        const int order[8] = {F_FO, F_FI, F_EO, F_EI, F_DH, F_KAP, F_LAP, F_MAG};
        for (int j = 0; j < 8; j++) memcpy(dbg + (size_t)j * n, F[order[j]], sizeof(float) * n);
    }
    free(buf);
    return 0;
}

/* T iterations of oracle_step_f32; phi is updated in place. */
int oracle_evolve_f32(float *phi, const float *I, int64_t W, int64_t H, int64_t L,
                      const oracle_params *p, int iters, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    size_t n = (size_t)W * H * L;
    float *tmp = (float *)malloc(sizeof(float) * n);
    if (!tmp) return -1;
    for (int t = 0; t < iters; t++) {
        int rc = oracle_step_f32(phi, I, tmp, W, H, L, p, NULL);
        if (rc) { free(tmp); return rc; }
        memcpy(phi, tmp, sizeof(float) * n);
    }
    free(tmp);
    return 0;
}

/* ======================================================================== */
/* FP64 twin: the same formulas evaluated entirely in double.               */
/* ======================================================================== */
static void diff_axis_d(const double *f, double *out, int64_t W, int64_t H, int64_t L,
                        int axis, int boundary) {
    int64_t n[3] = {W, H, L};
    int64_t st[3] = {1, W, W * H};
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < L; z++)
        for (int64_t y = 0; y < H; y++)
            for (int64_t x = 0; x < W; x++) {
                int64_t c[3] = {x, y, z};
                size_t i = idx3(x, y, z, W, H);
                int64_t pos = c[axis], N = n[axis];
                size_t il, ir;
                if (pos == 0) {
                    ir = i + (size_t)st[axis];
                    il = (axis == 0 && boundary == 0) ? (i > 0 ? i - 1 : 0) : i;
                } else if (pos == N - 1) {
                    ir = i;
                    il = i - (size_t)st[axis];
                } else {
                    ir = i + (size_t)st[axis];
                    il = i - (size_t)st[axis];
                }
                out[i] = (f[ir] - f[il]) / 2.0;
            }
}

static void conv_axis_d(const double *in, double *out, int64_t W, int64_t H, int64_t L,
                        int axis, const double *g, int k) {
    int64_t Wo = axis == 0 ? W - k + 1 : W, Ho = axis == 1 ? H - k + 1 : H, Lo = axis == 2 ? L - k + 1 : L;
    size_t st = axis == 0 ? 1 : axis == 1 ? (size_t)W : (size_t)W * H;
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < Lo; z++)
        for (int64_t y = 0; y < Ho; y++)
            for (int64_t x = 0; x < Wo; x++) {
                const double *src = in + idx3(x, y, z, W, H);
                double acc = 0.0;
                for (int t = 0; t < k; t++) acc += src[(size_t)t * st] * g[t];
                out[idx3(x, y, z, Wo, Ho)] = acc;
            }
}

static int blur_padded_d(const double *in, double *out, int64_t W, int64_t H, int64_t L,
                         const double *g, int k) {
    int64_t r = (k - 1) / 2;
    int64_t Wo = W - k + 1, Ho = H - k + 1, Lo = L - k + 1;
    size_t n = (size_t)W * H * L;
    if (Wo <= 0 || Ho <= 0 || Lo <= 0) {
        for (size_t i = 0; i < n; i++) out[i] = 30.0;
        return 0;
    }
    double *bx = (double *)malloc(sizeof(double) * (size_t)Wo * H * L);
    double *by = (double *)malloc(sizeof(double) * (size_t)Wo * Ho * L);
    double *bz = (double *)malloc(sizeof(double) * (size_t)Wo * Ho * Lo);
    if (!bx || !by || !bz) { free(bx); free(by); free(bz); return -1; }
    conv_axis_d(in, bx, W, H, L, 0, g, k);
    conv_axis_d(bx, by, Wo, H, L, 1, g, k);
    conv_axis_d(by, bz, Wo, Ho, L, 2, g, k);
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < L; z++)
        for (int64_t y = 0; y < H; y++)
            for (int64_t x = 0; x < W; x++) {
                int border = x < r || x >= Wo + r || y < r || y >= Ho + r || z < r || z >= Lo + r;
                out[idx3(x, y, z, W, H)] = border ? 30.0 : bz[idx3(x - r, y - r, z - r, Wo, Ho)];
            }
    free(bx); free(by); free(bz);
    return 0;
}

int oracle_step_f64(const double *phi, const float *I, double *phi_out,
                    int64_t W, int64_t H, int64_t L, const oracle_params *p) {
    float gf[512];
    double g[512];
    int k = oracle_taps(p->sigma, gf, 512);
    if (k < 0) return -2;
    for (int i = 0; i < k; i++) g[i] = gf[i];
    size_t n = (size_t)W * H * L;
    enum { D_HO, D_HI, D_IO, D_II, D_GX, D_GY, D_GZ, D_NX, D_NY, D_NZ, D_T0, D_T1, D_T2,
           D_KAP, D_LAP, D_BIO, D_BHO, D_BII, D_BHI, D_COUNT };
    double *buf = (double *)malloc(sizeof(double) * n * D_COUNT);
    if (!buf) return -1;
    double *F[D_COUNT];
    for (int i = 0; i < D_COUNT; i++) F[i] = buf + (size_t)i * n;
    double eps = p->eps;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        double h = 0.5 * (1.0 + (2.0 / RSF_PI) * atan(phi[i] / eps));
        F[D_HO][i] = h;
        F[D_HI][i] = 1.0 - h;
        F[D_IO][i] = (double)I[i] * h;
        F[D_II][i] = (double)I[i] * (1.0 - h);
    }
    diff_axis_d(phi, F[D_GX], W, H, L, 0, p->boundary);
    diff_axis_d(phi, F[D_GY], W, H, L, 1, p->boundary);
    diff_axis_d(phi, F[D_GZ], W, H, L, 2, p->boundary);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        double gx = F[D_GX][i], gy = F[D_GY][i], gz = F[D_GZ][i];
        double m = sqrt(gx * gx + gy * gy + gz * gz) + 1e-6;
        F[D_NX][i] = gx / m;
        F[D_NY][i] = gy / m;
        F[D_NZ][i] = gz / m;
    }
    diff_axis_d(F[D_NX], F[D_T0], W, H, L, 0, p->boundary);
    diff_axis_d(F[D_NY], F[D_T1], W, H, L, 1, p->boundary);
    diff_axis_d(F[D_NZ], F[D_T2], W, H, L, 2, p->boundary);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) F[D_KAP][i] = F[D_T0][i] + F[D_T1][i] + F[D_T2][i];
    diff_axis_d(F[D_GX], F[D_T0], W, H, L, 0, p->boundary);
    diff_axis_d(F[D_GY], F[D_T1], W, H, L, 1, p->boundary);
    diff_axis_d(F[D_GZ], F[D_T2], W, H, L, 2, p->boundary);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) F[D_LAP][i] = F[D_T0][i] + F[D_T1][i] + F[D_T2][i];
    int rc = 0;
    rc |= blur_padded_d(F[D_IO], F[D_BIO], W, H, L, g, k);
    rc |= blur_padded_d(F[D_HO], F[D_BHO], W, H, L, g, k);
    rc |= blur_padded_d(F[D_II], F[D_BII], W, H, L, g, k);
    rc |= blur_padded_d(F[D_HI], F[D_BHI], W, H, L, g, k);
    if (rc) { free(buf); return -1; }
    int s = (int)p->sigma2;
    double w = 1.0 / (double)((2 * s + 1) * (2 * s + 1));
    /* expanded Gaussian data term (data_term = 1): the blurs K*f, K*f^2 in
     * double, e = I^2 K*1 - 2 I K*f + K*f^2 on the valid region */
    double *kb = NULL, s3 = 0.0;
    int64_t r = (k - 1) / 2, Wo = W - k + 1, Ho = H - k + 1, Lo = L - k + 1;
    int gauss = p->data_term == 1 && Wo > 0 && Ho > 0 && Lo > 0;
    if (gauss) {
        double *fld = (double *)malloc(sizeof(double) * n);
        kb = (double *)malloc(sizeof(double) * n * 4);
        if (!fld || !kb) { free(fld); free(kb); free(buf); return -1; }
        for (int j = 0; j < 4; j++) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < (int64_t)n; i++) {
                double f = (j < 2) ? F[D_BIO][i] / F[D_BHO][i] : F[D_BII][i] / F[D_BHI][i];
                fld[i] = (j & 1) ? f * f : f;
            }
            if (blur_padded_d(fld, kb + (size_t)j * n, W, H, L, g, k)) { free(fld); free(kb); free(buf); return -1; }
        }
        free(fld);
        double sx = 0.0;
        for (int t = 0; t < k; t++) sx += g[t];
        s3 = sx * sx * sx;
    }
#pragma omp parallel for schedule(static)
    for (int64_t z = 0; z < L; z++)
        for (int64_t y = 0; y < H; y++)
            for (int64_t x = 0; x < W; x++) {
                size_t c = idx3(x, y, z, W, H);
                double fo = F[D_BIO][c] / F[D_BHO][c];
                double fi = F[D_BII][c] / F[D_BHI][c];
                double eo = 0.0, ei = 0.0;
                int inside = gauss && x >= r && x < Wo + r && y >= r && y < Ho + r && z >= r && z < Lo + r;
                if (inside) {
                    double Ic = I[c];
                    eo = Ic * Ic * s3 - 2.0 * Ic * kb[c] + kb[n + c];
                    ei = Ic * Ic * s3 - 2.0 * Ic * kb[2 * n + c] + kb[3 * n + c];
                } else for (int u = -s; u <= s; u++)
                    for (int v = -s; v <= s; v++)
                        for (int q = -s; q <= s; q++) {
                            int64_t yy = y + u, xx = x + v, zz = z + q;
                            if (yy < 0 || yy >= H || xx < 0 || xx >= W || zz < 0 || zz >= L) continue;
                            double In = I[idx3(xx, yy, zz, W, H)];
                            eo += w * (In - fo) * (In - fo);
                            ei += w * (In - fi) * (In - fi);
                        }
                double ph = phi[c];
                double dh = (1.0 / RSF_PI) * (eps / (eps * eps + ph * ph));
                double data = (double)p->lambda1 * eo - (double)p->lambda2 * ei;
                phi_out[c] = ph - dh * data * p->dt + (double)p->nu * p->dt * dh * F[D_KAP][c]
                             + (double)p->mu * p->dt * (F[D_LAP][c] - F[D_KAP][c]);
            }
    free(kb);
    free(buf);
    return 0;
}

int oracle_evolve_f64(double *phi, const float *I, int64_t W, int64_t H, int64_t L,
                      const oracle_params *p, int iters, int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    size_t n = (size_t)W * H * L;
    double *tmp = (double *)malloc(sizeof(double) * n);
    if (!tmp) return -1;
    for (int t = 0; t < iters; t++) {
        int rc = oracle_step_f64(phi, I, tmp, W, H, L, p);
        if (rc) { free(tmp); return rc; }
        memcpy(phi, tmp, sizeof(double) * n);
    }
    free(tmp);
    return 0;
}

/* Per-stage entries used by the unit tests. */
void oracle_heaviside(const float *phi, float *out, int64_t n, float eps, int arith) {
    for (int64_t i = 0; i < n; i++) out[i] = heaviside_f32(phi[i], eps, arith);
}
void oracle_dirac(const float *phi, float *out, int64_t n, float eps, int arith) {
    for (int64_t i = 0; i < n; i++) out[i] = dirac_f32(phi[i], eps, arith);
}
void oracle_normalise(const float *gx, const float *gy, const float *gz, float *nx, float *ny,
                      float *nz, float *mag, int64_t n, int form, int arith) {
    for (int64_t i = 0; i < n; i++) {
        float m = sqrtf(grad_mag2(gx[i], gy[i], gz[i], form));
        norm_den d = norm_den_make(m);
        mag[i] = m;
        nx[i] = normalise_f32(gx[i], m, &d, arith);
        ny[i] = normalise_f32(gy[i], m, &d, arith);
        nz[i] = normalise_f32(gz[i], m, &d, arith);
    }
}
/* Eout_Ein_calculation (kernel.cu:25-55) over given fits, box radius s. */
void oracle_data_terms(const float *I, const float *fo, const float *fi, float *eo, float *ei, int64_t W, int64_t H,
                       int64_t L, int s) {
    data_terms(I, fo, fi, eo, ei, W, H, L, s);
}
/* Final_phi (kernel.cu:365-387) over arrays, for stage-by-stage checks. */
void oracle_update_field(const float *phi, const float *dh, const float *eo, const float *ei, const float *kap,
                         const float *lap, float *out, int64_t n, const oracle_params *p) {
    for (int64_t i = 0; i < n; i++) out[i] = update_f32(phi[i], dh[i], eo[i], ei[i], kap[i], lap[i], p);
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/*
 * Initial level set (CUDA_RSF/main.cpp:174-183: phi0 = sdf(seed - 13)).  The
 * reference's sdf() is tiralib's (third party, not in the reference
 * checkout), so this restates the definition the GPU implements, not an
 * algorithm of the reference: inside = seed > threshold; phi0 = +d(p, outside)
 * at inside voxels and -d(p, inside) at outside voxels, d Euclidean between
 * voxel centres; +-(W+H+L) when the other class is empty.  Computed by
 * direct minimisation: squared distances along x by scanning the row, then
 * D(y) = min_y' (D(y') + (y-y')^2) over each column and likewise along z, in
 * exact 64-bit integers (O(n^2) per line: small volumes only).
 */
static void sdf_class(const float *seed, float thr, int feat_inside, float *phi, int64_t W, int64_t H,
                      int64_t L, uint64_t *d, uint64_t *col) {
    const uint64_t INF = ~(uint64_t)0;
    for (int64_t z = 0; z < L; z++)
        for (int64_t y = 0; y < H; y++)
            for (int64_t x = 0; x < W; x++) {
                uint64_t best = INF;
                for (int64_t u = 0; u < W; u++) {
                    if ((seed[idx3(u, y, z, W, H)] > thr) != (feat_inside != 0)) continue;
                    uint64_t dd = (uint64_t)((u - x) * (u - x));
                    if (dd < best) best = dd;
                }
                d[idx3(x, y, z, W, H)] = best;
            }
    for (int axis = 1; axis <= 2; axis++) {
        const int64_t n = axis == 1 ? H : L;
        for (int64_t a = 0; a < (axis == 1 ? L : H); a++)
            for (int64_t x = 0; x < W; x++) {
                for (int64_t q = 0; q < n; q++) {
                    uint64_t best = INF;
                    for (int64_t v = 0; v < n; v++) {
                        const uint64_t f = axis == 1 ? d[idx3(x, v, a, W, H)] : d[idx3(x, a, v, W, H)];
                        if (f == INF) continue;
                        const uint64_t c = f + (uint64_t)((q - v) * (q - v));
                        if (c < best) best = c;
                    }
                    col[q] = best;
                }
                for (int64_t q = 0; q < n; q++) {
                    if (axis == 1) d[idx3(x, q, a, W, H)] = col[q];
                    else d[idx3(x, a, q, W, H)] = col[q];
                }
            }
    }
    const float fill = (float)W + (float)H + (float)L;
    for (int64_t i = 0; i < W * H * L; i++) {
        if ((seed[i] > thr) == (feat_inside != 0)) continue;
        const float mag = d[i] == INF ? fill : sqrtf((float)d[i]);
        phi[i] = feat_inside ? -mag : mag;
    }
}

int oracle_signed_distance(const float *seed, float thr, float *phi, int64_t W, int64_t H, int64_t L) {
    if (W < 1 || H < 1 || L < 1) return 1;
    const int64_t n = W * H * L;
    int64_t m = W > H ? W : H;
    if (L > m) m = L;
    uint64_t *d = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n);
    uint64_t *col = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)m);
    if (!d || !col) { free(d); free(col); return 2; }
    sdf_class(seed, thr, 0, phi, W, H, L, d, col);
    sdf_class(seed, thr, 1, phi, W, H, L, d, col);
    free(d);
    free(col);
    return 0;
}
