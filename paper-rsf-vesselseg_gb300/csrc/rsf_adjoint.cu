// rsf_adjoint.cu -- reverse-mode derivative of one RSF step, for a batch of
// volumes that share the step parameters.
//
// The forward step (CUDA_RSF/main.cpp:233-300, kernel.cu) maps phi to
//   phi' = phi + dt * ( -delta(phi) * data + nu * delta(phi) * kappa + mu * (Lap - kappa) )
// with data = lambda1 * e_out - lambda2 * e_in, e = (I - f)^2, f the ratios of
// Gaussian-blurred fields (I H, H, I (1-H), 1-H), kappa = sum_a D_a n_a,
// n = g / (|g| + 1e-6), g_a = D_a phi, Lap = sum_a D_a D_a phi, and D_a the
// central difference with the reference's boundary rules (kernel.cu:57-125).
// Given u = dL/dphi', this file computes dL/dphi and accumulates dL/dlambda1,
// dL/dlambda2, dL/dmu, dL/dnu.  The derivative is that of the exact real
// function above (H' = delta; delta' = -2 phi delta / (eps^2 + phi^2)), evaluated
// in FP32; it is not the derivative of the floating-point rounding.
//
// Chain, with pointwise adjoints written as bars:
//   data_bar  = -u dt delta       e_out_bar = lambda1 data_bar, e_in_bar = -lambda2 data_bar
//   f_bar     = -2 (I - f) e_bar  (valid region only; the border band holds f = 1)
//   B1_bar = f_out_bar / B2, B2_bar = -f_out_bar f_out / B2 (and B3, B4 from f_in)
//   H_bar  = I * G^T (B1_bar - B3_bar) + G^T (B2_bar - B4_bar)    (blur is linear)
//   kappa_bar = u dt (nu delta - mu), Lap_bar = u dt mu
//   n_bar_a = D_a^T kappa_bar;  g_bar_a = D_a^T Lap_bar + (n_bar_a - (n_bar . n) g_a/|g|) / (|g| + 1e-6)
//   phi_bar = u + delta H_bar + delta' u dt (-data + nu kappa) + sum_a D_a^T g_bar_a
// G^T of the valid correlation is the full correlation with the same
// (symmetric) taps.  D_a^T is gathered: voxel j collects 0.5 v(m) for every m
// among its three axis neighbours whose right index is j, and -0.5 v(m) for
// every m whose left index is j, so boundary rules transpose exactly.
//
// Kernels: H; blur recompute x, y, z (the z kernel also forms the data-term
// adjoint); transposed blur z, y, x (the x kernel forms H_bar); gradients and
// unit normals; the pointwise terms with the parameter sums; the stencil
// adjoint w; the final D^T gather.  The blurs along y and z compute several
// consecutive outputs per thread; the last three kernels run on blocks of
// 32 x 8 voxels, the others on one item per thread.  Every kernel covers the
// whole batch in one launch: a block finds its volume in a block prefix
// array (one per kernel) and its tile within the volume.  For 21, 29 and 35
// taps the caller replaces the first four kernels by the forward step's
// streaming x- and y-passes and the z-pass's adjoint variant
// (zpass_adjoint_kernel), which leave the same fields in xs.
//
// Scratch per volume (N = W H L; slices of the workspace pools of 1, 4 and
// 4 floats per voxel):
//   phi2 : H (blur input), later H_bar
//   xs   : blur-x fields (4 Wv H L), then [0, 2N) the valid-layout adjoint pair
//          and [2N, 4N) e_out, e_in (kappa_bar over e_out); then g_x, g_y in
//          [0, 2N), later w_x, w_y
//   ys   : blur-y fields (4 Wv Hv L), then the z-transposed pair [0, 2N), the
//          y-transposed pair at 2N; later g_z (then w_z), n_x, n_y, n_z
#include <cuda_runtime.h>

#include "rsf_arith.cuh"
#include "rsf_internal.h"

namespace rsf {
namespace {

constexpr int kThreads = 256;

struct AdjConst {
    float taps[MAXK];
    int k, r;
    float eps, dt, mu, nu, l1, l2;
    int boundary;    // 0 reference (x = 0 reads the previous linear element), 1 clamp
    int img_f32;
    int nvol;
};

__device__ __forceinline__ float img_at(const void *img, long long i, int f32) {
    return f32 ? static_cast<const float *>(img)[i] : (float)static_cast<const unsigned char *>(img)[i];
}

// The volume of this block (binary search of the kernel's block prefix
// array) and the block's index within it.  Kernels copy their volume's
// descriptor by value, so that their stores cannot alias it and its fields
// are loaded once.
struct BlockVol {
    int v;
    long long t;
};
__device__ __forceinline__ BlockVol block_vol(const int *__restrict__ pre, int n) {
    const int b = blockIdx.x;
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(pre + mid) <= b) lo = mid;
        else hi = mid;
    }
    return {lo, (long long)(b - __ldg(pre + lo))};
}

// The stencil kernels run on blocks of 32 x 8 voxels of kWZ planes (w,
// gather) or of kPointZ planes (pointwise terms).
constexpr int kBX = 32, kBY = 8;
constexpr int kPointZ = 16;
constexpr int kWZ = 8;  // planes per block of adj_w and adj_gather

struct Geo {
    int W, H, L, boundary;
};

// Right and left linear indices of the central difference at voxel i.
__device__ __forceinline__ void nb_x(const Geo &g, long long i, int x, long long &r, long long &l) {
    r = x + 1 < g.W ? i + 1 : i;
    if (x > 0) l = i - 1;
    else l = g.boundary == 0 ? (i > 0 ? i - 1 : 0) : i;
    if (x == g.W - 1) l = i - 1;
}
// y and z: (f[1] - f[0]) / 2 at 0, (f[n-1] - f[n-2]) / 2 at n - 1 (n >= 2).
__device__ __forceinline__ void nb_axis(long long i, int q, int n, long long stride, long long &r, long long &l) {
    const int qr = q + 1 < n ? q + 1 : n - 1;
    const int ql = q > 0 ? q - 1 : 0;
    r = i + (long long)(qr - q) * stride;
    l = i + (long long)(ql - q) * stride;
}

__device__ __forceinline__ float diff_x_at(const Geo &g, const float *f, long long m, int x) {
    long long r, l;
    nb_x(g, m, x, r, l);
    return 0.5f * (f[r] - f[l]);
}
__device__ __forceinline__ float diff_axis_at(const float *f, long long m, int q, int n, long long stride) {
    long long r, l;
    nb_axis(m, q, n, stride, r, l);
    return 0.5f * (f[r] - f[l]);
}

// (D_x^T v)(j): the neighbours j-1, j, j+1 in linear order are the only
// voxels whose difference reads j.
// x is j's x coordinate; the linear neighbours of a row's end are the next
// row's start and vice versa.  Branch-free: an out-of-range candidate is
// read as j itself with coefficient 0, so that all loads issue together.
template <class V>
__device__ __forceinline__ float dT_x(const Geo &g, long long j, int x, long long N, V v) {
    float acc = 0.0f;
#pragma unroll
    for (int d = -1; d <= 1; d++) {
        const long long m0 = j + d;
        const bool in = m0 >= 0 && m0 < N;
        const long long m = in ? m0 : j;
        const int mx = d == 0 ? x : d < 0 ? (x > 0 ? x - 1 : g.W - 1) : (x + 1 < g.W ? x + 1 : 0);
        long long r, l;
        nb_x(g, m, mx, r, l);
        const float coef = in ? (r == j ? 0.5f : 0.0f) - (l == j ? 0.5f : 0.0f) : 0.0f;
        acc = fmaf(coef, v(m), acc);
    }
    return acc;
}
template <class V>
__device__ __forceinline__ float dT_axis(long long j, int q, int n, long long stride, V v) {
    float acc = 0.0f;
#pragma unroll
    for (int d = -1; d <= 1; d++) {
        const bool in = q + d >= 0 && q + d < n;
        const int qm = in ? q + d : q;
        const long long m = j + (long long)(qm - q) * stride;
        long long r, l;
        nb_axis(m, qm, n, stride, r, l);
        const float coef = in ? (r == j ? 0.5f : 0.0f) - (l == j ? 0.5f : 0.0f) : 0.0f;
        acc = fmaf(coef, v(m), acc);
    }
    return acc;
}

// D_a^T v at a voxel that is neither first nor last along any axis: only
// j - s (coefficient 1/2) and j + s (-1/2) read j, as in dT_x / dT_axis,
// whose evaluation order this keeps (the coefficient-0 term of j itself
// adds nothing to a finite sum).
template <class V>
__device__ __forceinline__ float dT_in(long long j, long long s, V v) {
    return fmaf(-0.5f, v(j + s), 0.5f * v(j - s));
}

// The voxel is neither first nor last along any axis (the x = 0 and last-index
// rules of the differences and of their transposes do not apply).
__device__ __forceinline__ bool inner_voxel(const AdjVol &a, int x, int y, int z) {
    return x >= 1 && x <= a.W - 2 && y >= 1 && y <= a.H - 2 && z >= 1 && z <= a.L - 2;
}

// delta(phi) with a fast division: the adjoint needs the derivative's value,
// not the forward's bit pattern.
__device__ __forceinline__ float dirac_fast(float phi, float eps) {
    return __fdividef(0.318309886183790672f * eps, fmaf(phi, phi, eps * eps));
}

__device__ __forceinline__ long long nvox(const AdjVol &a) { return (long long)a.W * a.H * a.L; }
__device__ __forceinline__ long long item(const BlockVol &bv) { return bv.t * kThreads + threadIdx.x; }

__global__ void __launch_bounds__(kThreads) adj_heaviside(AdjConst c, const AdjVol *__restrict__ vols,
                                                          const int *__restrict__ pre) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long i = item(bv);
    if (i < nvox(a)) a.phi2[i] = heaviside<Arith::Portable>(a.phi[i], c.eps);
}

// Valid correlation along x of (I H, H, I (1-H), 1-H): (Wv, H, L) per field,
// from H in phi2 to xs.
__global__ void __launch_bounds__(kThreads) adj_blur_x(AdjConst c, const AdjVol *__restrict__ vols,
                                                       const int *__restrict__ pre) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long n = (long long)a.Wv * a.H * a.L;
    const long long o = item(bv);
    if (o >= n) return;
    const int xv = (int)(o % a.Wv);
    const long long row = o / a.Wv;  // z * H + y
    const long long base = row * a.W + xv;
    const float *h = a.phi2;
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    for (int t = 0; t < c.k; t++) {
        const float hv = h[base + t];
        const float I = img_at(a.img, base + t, c.img_f32);
        const float hi = 1.0f - hv;
        const float g = c.taps[t];
        a0 = fmaf(I * hv, g, a0);
        a1 = fmaf(hv, g, a1);
        a2 = fmaf(I * hi, g, a2);
        a3 = fmaf(hi, g, a3);
    }
    float *out = a.xs;
    out[o] = a0;
    out[n + o] = a1;
    out[2 * n + o] = a2;
    out[3 * n + o] = a3;
}

// Correlation of NB consecutive outputs start .. start+NB-1 along a strided
// axis of nin inputs, register-blocked so that each input load feeds up to
// NB outputs.  Valid: out[o] = sum_t g[t] in[o + t].  Transposed (the
// adjoint of valid): out[o] = sum_t g[t] in[o - t] over 0 <= o - t < nin.
template <int NB, bool TRANSPOSED>
__device__ __forceinline__ void corr_block(const AdjConst &c, const float *__restrict__ col, long long stride,
                                           int start, int nin, float (&acc)[NB]) {
#pragma unroll
    for (int m = 0; m < NB; ++m) acc[m] = 0.0f;
    const int p0 = TRANSPOSED ? start - c.k + 1 : start;
    const int p1 = TRANSPOSED ? start + NB : start + NB + c.k - 1;  // exclusive
    for (int p = max(p0, 0); p < min(p1, nin); ++p) {
        const float v = col[(long long)p * stride];
#pragma unroll
        for (int m = 0; m < NB; ++m) {
            const int t = TRANSPOSED ? start + m - p : p - start - m;
            if (t >= 0 && t < c.k) acc[m] = fmaf(v, c.taps[t], acc[m]);
        }
    }
}

constexpr int kNB = 8;   // outputs per thread along z
constexpr int kNBy = 4;  // outputs per thread along y (shorter columns keep more threads in flight)

// Valid correlation along y: xs (Wv, H, L) -> ys (Wv, Hv, L), four fields.
__global__ void __launch_bounds__(kThreads) adj_blur_y(AdjConst c, const AdjVol *__restrict__ vols,
                                                       const int *__restrict__ pre) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long nin = (long long)a.Wv * a.H * a.L, n = (long long)a.Wv * a.Hv * a.L;
    const int nyb = (a.Hv + kNBy - 1) / kNBy;
    const long long q = item(bv);
    if (q >= (long long)a.Wv * nyb * a.L) return;
    const int xv = (int)(q % a.Wv);
    const long long t1 = q / a.Wv;
    const int y0 = (int)(t1 % nyb) * kNBy;
    const int z = (int)(t1 / nyb);
    for (int f = 0; f < 4; f++) {
        float acc[kNBy];
        corr_block<kNBy, false>(c, a.xs + f * nin + (long long)z * a.H * a.Wv + xv, a.Wv, y0, a.H, acc);
#pragma unroll
        for (int m = 0; m < kNBy; ++m)
            if (y0 + m < a.Hv) a.ys[f * n + ((long long)z * a.Hv + y0 + m) * a.Wv + xv] = acc[m];
    }
}

// Valid correlation along z, then the data-term adjoint at each valid voxel:
// writes (B1_bar - B3_bar, B2_bar - B4_bar) in the valid layout to xs and
// e_out, e_in at the full-volume index to xs + 2N, xs + 3N.
__global__ void __launch_bounds__(kThreads) adj_blur_z_data(AdjConst c, const AdjVol *__restrict__ vols,
                                                            const int *__restrict__ pre) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long N = nvox(a);
    const long long nin = (long long)a.Wv * a.Hv * a.L, n = (long long)a.Wv * a.Hv * a.Lv;
    const long long plane = (long long)a.Wv * a.Hv;
    const int nzb = (a.Lv + kNB - 1) / kNB;
    const long long q = item(bv);
    if (q >= plane * nzb) return;
    const long long pxy = q % plane;
    const int z0 = (int)(q / plane) * kNB;
    const int xv = (int)(pxy % a.Wv), yv = (int)(pxy / a.Wv);
    float B[4][kNB];
    for (int f = 0; f < 4; f++) corr_block<kNB, false>(c, a.ys + f * nin + pxy, plane, z0, a.L, B[f]);
    float *pq = a.xs, *eo_out = a.xs + 2 * N, *ei_out = a.xs + 3 * N;
#pragma unroll
    for (int m = 0; m < kNB; ++m) {
        const int zv = z0 + m;
        if (zv >= a.Lv) break;
        const long long o = (long long)zv * plane + pxy;
        const long long i = ((long long)(zv + c.r) * a.H + (yv + c.r)) * a.W + xv + c.r;
        const float I = img_at(a.img, i, c.img_f32);
        const float rb1 = __frcp_rn(B[1][m]), rb3 = __frcp_rn(B[3][m]);
        const float fo = B[0][m] * rb1, fi = B[2][m] * rb3;
        const float dfo = I - fo, dfi = I - fi;
        eo_out[i] = dfo * dfo;
        ei_out[i] = dfi * dfi;
        const float delta = dirac_fast(a.phi[i], c.eps);
        const float data_bar = -a.u[i] * c.dt * delta;
        const float fo_bar = -2.0f * dfo * (c.l1 * data_bar);
        const float fi_bar = -2.0f * dfi * (-c.l2 * data_bar);
        const float b1 = fo_bar * rb1, b2 = -fo_bar * fo * rb1;
        const float b3 = fi_bar * rb3, b4 = -fi_bar * fi * rb3;
        pq[o] = b1 - b3;
        pq[n + o] = b2 - b4;
    }
}

// Transposed (full) correlation along z: xs (Wv, Hv, Lv) -> ys (Wv, Hv, L), two fields.
__global__ void __launch_bounds__(kThreads) adj_blurT_z(AdjConst c, const AdjVol *__restrict__ vols,
                                                        const int *__restrict__ pre) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long nin = (long long)a.Wv * a.Hv * a.Lv, n = (long long)a.Wv * a.Hv * a.L;
    const long long plane = (long long)a.Wv * a.Hv;
    const int nzb = (a.L + kNB - 1) / kNB;
    const long long q = item(bv);
    if (q >= plane * nzb) return;
    const long long pxy = q % plane;
    const int z0 = (int)(q / plane) * kNB;
    for (int f = 0; f < 2; f++) {
        float acc[kNB];
        corr_block<kNB, true>(c, a.xs + f * nin + pxy, plane, z0, a.Lv, acc);
#pragma unroll
        for (int m = 0; m < kNB; ++m)
            if (z0 + m < a.L) a.ys[f * n + (long long)(z0 + m) * plane + pxy] = acc[m];
    }
}

// Transposed correlation along y: ys (Wv, Hv, L) -> ys + 2N (Wv, H, L).
__global__ void __launch_bounds__(kThreads) adj_blurT_y(AdjConst c, const AdjVol *__restrict__ vols,
                                                        const int *__restrict__ pre) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long nin = (long long)a.Wv * a.Hv * a.L, n = (long long)a.Wv * a.H * a.L;
    const int nyb = (a.H + kNBy - 1) / kNBy;
    const long long q = item(bv);
    if (q >= (long long)a.Wv * nyb * a.L) return;
    const int xv = (int)(q % a.Wv);
    const long long t1 = q / a.Wv;
    const int y0 = (int)(t1 % nyb) * kNBy;
    const int z = (int)(t1 / nyb);
    float *out = a.ys + 2 * nvox(a);
    for (int f = 0; f < 2; f++) {
        float acc[kNBy];
        corr_block<kNBy, true>(c, a.ys + f * nin + (long long)z * a.Hv * a.Wv + xv, a.Wv, y0, a.Hv, acc);
#pragma unroll
        for (int m = 0; m < kNBy; ++m)
            if (y0 + m < a.H) out[f * n + ((long long)z * a.H + y0 + m) * a.Wv + xv] = acc[m];
    }
}

// Transposed correlation along x and H_bar = I * P~ + Q~ over the volume,
// into phi2 (0 for a volume without a valid region).
__global__ void __launch_bounds__(kThreads) adj_blurT_x_hbar(AdjConst c, const AdjVol *__restrict__ vols,
                                                             const int *__restrict__ pre) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long N = nvox(a);
    const long long nin = (long long)a.Wv * a.H * a.L;
    const long long i = item(bv);
    if (i >= N) return;
    if (a.Wv == 0) {
        a.phi2[i] = 0.0f;
        return;
    }
    const float *in = a.ys + 2 * N;
    const int x = (int)(i % a.W);
    const long long row = i / a.W;
    const int a0 = max(0, x - a.Wv + 1), a1 = min(c.k - 1, x);
    float p = 0.0f, q = 0.0f;
    for (int t = a0; t <= a1; t++) {
        const long long s = row * a.Wv + (x - t);
        p = fmaf(in[s], c.taps[t], p);
        q = fmaf(in[nin + s], c.taps[t], q);
    }
    a.phi2[i] = fmaf(img_at(a.img, i, c.img_f32), p, q);
}

// Gradient g = D phi and unit normals n = g / (|g| + 1e-6), stored so that
// the stencil adjoint reads them at its neighbours instead of recomputing:
// g_x, g_y to xs, xs + N; g_z, n_x, n_y, n_z to ys .. ys + 3N.
__global__ void __launch_bounds__(kThreads) adj_normals(AdjConst c, const AdjVol *__restrict__ vols,
                                                        const int *__restrict__ pre) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long N = nvox(a);
    const long long i = item(bv);
    if (i >= N) return;
    const Geo g = {a.W, a.H, a.L, c.boundary};
    const int x = (int)(i % a.W);
    const long long t1 = i / a.W;
    const int y = (int)(t1 % a.H);
    const int z = (int)(t1 / a.H);
    const long long plane = (long long)a.W * a.H;
    float gx, gy, gz;
    if (inner_voxel(a, x, y, z)) {
        gx = 0.5f * (a.phi[i + 1] - a.phi[i - 1]);
        gy = 0.5f * (a.phi[i + a.W] - a.phi[i - a.W]);
        gz = 0.5f * (a.phi[i + plane] - a.phi[i - plane]);
    } else {
        gx = diff_x_at(g, a.phi, i, x);
        gy = diff_axis_at(a.phi, i, y, a.H, a.W);
        gz = diff_axis_at(a.phi, i, z, a.L, plane);
    }
    const float rs = __frcp_rn(sqrtf(gx * gx + gy * gy + gz * gz) + 1e-6f);
    a.xs[i] = gx;
    a.xs[N + i] = gy;
    a.ys[i] = gz;
    a.ys[N + i] = gx * rs;
    a.ys[2 * N + i] = gy * rs;
    a.ys[3 * N + i] = gz * rs;
}

// The block's 32 x 8 column: x, y of this thread and the first z plane.
struct Col {
    int x, y, z0;
};
__device__ __forceinline__ Col col_of(const AdjVol &a, long long t, int zdepth) {
    const int nbx = (a.W + kBX - 1) / kBX, nby = (a.H + kBY - 1) / kBY;
    const long long t1 = t / nbx;
    return {(int)(t % nbx) * kBX + (int)threadIdx.x, (int)(t1 % nby) * kBY + (int)threadIdx.y,
            (int)(t1 / nby) * zdepth};
}

// Pointwise terms and parameter sums:
//   out = u + delta H_bar + delta' u dt (nu kappa - data),
// with kappa = sum_a D_a n_a and Lap = sum_a D_a g_a from the stored fields.
// A block covers a 32 x 8 column of kPointZ planes; the parameter sums are
// reduced in the block and added with one double atomic per parameter and
// block (the same four addresses for every block, so their number matters).
// kappa_bar = u dt (nu delta - mu) is written over e_out (read first, by the
// same thread) for adj_w.
__global__ void __launch_bounds__(kBX * kBY) adj_point(AdjConst c, const AdjVol *__restrict__ vols,
                                                       const int *__restrict__ pre,
                                                       double *grads) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long N = nvox(a);
    const long long plane = (long long)a.W * a.H;
    const Geo g = {a.W, a.H, a.L, c.boundary};
    const float *gxa = a.xs, *gya = a.xs + N, *gza = a.ys;
    const float *nx = a.ys + N, *ny = a.ys + 2 * N, *nz = a.ys + 3 * N;
    float *eo_v = a.xs + 2 * N;
    const float *ei_v = a.xs + 3 * N;
    float s_l1 = 0.0f, s_l2 = 0.0f, s_mu = 0.0f, s_nu = 0.0f;
    const Col cl = col_of(a, bv.t, kPointZ);
    const int x = cl.x, y = cl.y;
    const int z1 = min(cl.z0 + kPointZ, a.L);
    for (int z = cl.z0; z < z1 && x < a.W && y < a.H; ++z) {
        const long long i = ((long long)z * a.H + y) * a.W + x;
        const float ph = a.phi[i], ui = a.u[i];
        const float I = img_at(a.img, i, c.img_f32);
        const float delta = dirac_fast(ph, c.eps);
        const float ddelta = __fdividef(-2.0f * ph * delta, fmaf(ph, ph, c.eps * c.eps));
        long long rx, lx, ry, ly, rz, lz;
        nb_x(g, i, x, rx, lx);
        nb_axis(i, y, a.H, a.W, ry, ly);
        nb_axis(i, z, a.L, plane, rz, lz);
        const float kap = 0.5f * (nx[rx] - nx[lx]) + 0.5f * (ny[ry] - ny[ly]) + 0.5f * (nz[rz] - nz[lz]);
        const float lap = 0.5f * (gxa[rx] - gxa[lx]) + 0.5f * (gya[ry] - gya[ly]) + 0.5f * (gza[rz] - gza[lz]);
        const bool valid = a.Wv > 0 && x >= c.r && x < c.r + a.Wv && y >= c.r && y < c.r + a.Hv && z >= c.r &&
                           z < c.r + a.Lv;
        float eo, ei;
        if (valid) {
            eo = eo_v[i];
            ei = ei_v[i];
        } else {  // border band: f_out = f_in = 30 / 30
            eo = ei = (I - 1.0f) * (I - 1.0f);
        }
        const float data = c.l1 * eo - c.l2 * ei;
        a.out[i] = ui + delta * a.phi2[i] + ddelta * ui * c.dt * (c.nu * kap - data);
        const float ud = ui * c.dt, udd = ud * delta;
        eo_v[i] = ud * (c.nu * delta - c.mu);
        s_l1 = fmaf(-udd, eo, s_l1);
        s_l2 = fmaf(udd, ei, s_l2);
        s_mu = fmaf(ud, lap - kap, s_mu);
        s_nu = fmaf(udd, kap, s_nu);
    }
    if (grads) {  // uniform: every thread reaches the shuffles and the barrier
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s_l1 += __shfl_down_sync(0xffffffffu, s_l1, o);
            s_l2 += __shfl_down_sync(0xffffffffu, s_l2, o);
            s_mu += __shfl_down_sync(0xffffffffu, s_mu, o);
            s_nu += __shfl_down_sync(0xffffffffu, s_nu, o);
        }
        __shared__ float part[kBY][4];
        if (threadIdx.x == 0) {
            part[threadIdx.y][0] = s_l1;
            part[threadIdx.y][1] = s_l2;
            part[threadIdx.y][2] = s_mu;
            part[threadIdx.y][3] = s_nu;
        }
        __syncthreads();
        if (threadIdx.y == 0 && threadIdx.x < 4) {
            double acc = 0.0;
            for (int w = 0; w < kBY; ++w) acc += (double)part[w][threadIdx.x];
            atomicAdd(grads + threadIdx.x, acc);
        }
    }
}

// Stencil adjoint: w_a = D_a^T Lap_bar + (n_bar_a - (n_bar . n) g_a/|g|) / (|g| + 1e-6)
// with n_bar = D^T kappa_bar, to be gathered by D_a^T.  kappa_bar comes from
// adj_point; Lap_bar = u dt mu.  Each thread reads g and n at its own voxel
// only, so w is written over g in place.
__global__ void __launch_bounds__(kBX * kBY) adj_w(AdjConst c, const AdjVol *__restrict__ vols,
                                                   const int *__restrict__ pre) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long N = nvox(a);
    const long long plane = (long long)a.W * a.H;
    const Geo g = {a.W, a.H, a.L, c.boundary};
    const float *kb = a.xs + 2 * N, *u = a.u;
    auto kbar = [&](long long m) { return kb[m]; };
    auto lbar = [&](long long m) { return u[m] * c.dt * c.mu; };
    const Col cl = col_of(a, bv.t, kWZ);
    const int x = cl.x, y = cl.y;
    const int z1 = min(cl.z0 + kWZ, a.L);
    for (int z = cl.z0; z < z1 && x < a.W && y < a.H; ++z) {
        float *gxa = a.xs, *gya = a.xs + N, *gza = a.ys;
        const float *nx = a.ys + N, *ny = a.ys + 2 * N, *nz = a.ys + 3 * N;
        const long long i = ((long long)z * a.H + y) * a.W + x;
        const float gx = gxa[i], gy = gya[i], gz = gza[i];
        const float mag = sqrtf(gx * gx + gy * gy + gz * gz);
        const float rs = __frcp_rn(mag + 1e-6f);
        const float inv_mag = mag > 0.0f ? __frcp_rn(mag) : 0.0f;
        float nbx, nby, nbz, lbx, lby, lbz;
        if (inner_voxel(a, x, y, z)) {
            nbx = dT_in(i, 1, kbar);
            nby = dT_in(i, a.W, kbar);
            nbz = dT_in(i, plane, kbar);
            lbx = dT_in(i, 1, lbar);
            lby = dT_in(i, a.W, lbar);
            lbz = dT_in(i, plane, lbar);
        } else {
            nbx = dT_x(g, i, x, N, kbar);
            nby = dT_axis(i, y, a.H, a.W, kbar);
            nbz = dT_axis(i, z, a.L, plane, kbar);
            lbx = dT_x(g, i, x, N, lbar);
            lby = dT_axis(i, y, a.H, a.W, lbar);
            lbz = dT_axis(i, z, a.L, plane, lbar);
        }
        const float ndot = nbx * nx[i] + nby * ny[i] + nbz * nz[i];
        gxa[i] = lbx + (nbx - ndot * gx * inv_mag) * rs;
        gya[i] = lby + (nby - ndot * gy * inv_mag) * rs;
        gza[i] = lbz + (nbz - ndot * gz * inv_mag) * rs;
    }
}

// out += sum_a D_a^T w_a; a non-finite result sets kFlagAdjointNonFinite.
__global__ void __launch_bounds__(kBX * kBY) adj_gather(AdjConst c, const AdjVol *__restrict__ vols,
                                                        const int *__restrict__ pre, unsigned *flag) {
    const BlockVol bv = block_vol(pre, c.nvol);
    const AdjVol a = vols[bv.v];
    const long long N = nvox(a);
    const long long plane = (long long)a.W * a.H;
    const Geo g = {a.W, a.H, a.L, c.boundary};
    const float *wx = a.xs, *wy = a.xs + N, *wz = a.ys;
    auto vx = [&](long long m) { return wx[m]; };
    auto vy = [&](long long m) { return wy[m]; };
    auto vz = [&](long long m) { return wz[m]; };
    const Col cl = col_of(a, bv.t, kWZ);
    const int x = cl.x, y = cl.y;
    const int z1 = min(cl.z0 + kWZ, a.L);
    for (int z = cl.z0; z < z1 && x < a.W && y < a.H; ++z) {
        const long long i = ((long long)z * a.H + y) * a.W + x;
        const float d = inner_voxel(a, x, y, z)
                            ? dT_in(i, 1, vx) + dT_in(i, a.W, vy) + dT_in(i, plane, vz)
                            : dT_x(g, i, x, N, vx) + dT_axis(i, y, a.H, a.W, vy) + dT_axis(i, z, a.L, plane, vz);
        const float v = a.out[i] + d;
        a.out[i] = v;
        if (!isfinite(v) && flag) atomicOr(flag, kFlagAdjointNonFinite);
    }
}

long long cdiv(long long a, long long b) { return (a + b - 1) / b; }

}  // namespace

void adjoint_tiles(const AdjVol &v, bool streamed, int tiles[NADJ]) {
    const long long N = (long long)v.W * v.H * v.L;
    const bool valid = v.Wv > 0;
    const long long bxy = cdiv(v.W, kBX) * cdiv(v.H, kBY);
    long long t[NADJ] = {};
    if (valid) {
        if (!streamed) {
            t[ADJ_H] = cdiv(N, kThreads);
            t[ADJ_BX] = cdiv((long long)v.Wv * v.H * v.L, kThreads);
            t[ADJ_BY] = cdiv((long long)v.Wv * cdiv(v.Hv, kNBy) * v.L, kThreads);
            t[ADJ_BZ] = cdiv((long long)v.Wv * v.Hv * cdiv(v.Lv, kNB), kThreads);
        }
        t[ADJ_TZ] = cdiv((long long)v.Wv * v.Hv * cdiv(v.L, kNB), kThreads);
        t[ADJ_TY] = cdiv((long long)v.Wv * cdiv(v.H, kNBy) * v.L, kThreads);
    }
    t[ADJ_TX] = cdiv(N, kThreads);
    t[ADJ_NRM] = cdiv(N, kThreads);
    t[ADJ_PT] = bxy * cdiv(v.L, kPointZ);
    t[ADJ_W] = bxy * cdiv(v.L, kWZ);
    t[ADJ_G] = bxy * cdiv(v.L, kWZ);
    for (int j = 0; j < NADJ; j++) tiles[j] = t[j] > 0x7fffffffLL ? -1 : (int)t[j];
}

cudaError_t launch_step_adjoint(const float *taps, int k, const AdjScalars &s, const AdjVol *vols, const int *pre,
                                int n, const int *tot, double *grads, unsigned *flag, cudaStream_t st) {
    AdjConst c;
    for (int t = 0; t < MAXK; t++) c.taps[t] = t < k ? taps[t] : 0.0f;
    c.k = k;
    c.r = (k - 1) / 2;
    c.eps = s.eps;
    c.dt = s.dt;
    c.mu = s.mu;
    c.nu = s.nu;
    c.l1 = s.l1;
    c.l2 = s.l2;
    c.boundary = s.boundary;
    c.img_f32 = s.img_f32;
    c.nvol = n;
    const int n1 = n + 1;
    auto P = [&](int j) { return pre + (size_t)j * n1; };
    const dim3 b2(kBX, kBY, 1);
    if (tot[ADJ_H] > 0) adj_heaviside<<<tot[ADJ_H], kThreads, 0, st>>>(c, vols, P(ADJ_H));
    if (tot[ADJ_BX] > 0) adj_blur_x<<<tot[ADJ_BX], kThreads, 0, st>>>(c, vols, P(ADJ_BX));
    if (tot[ADJ_BY] > 0) adj_blur_y<<<tot[ADJ_BY], kThreads, 0, st>>>(c, vols, P(ADJ_BY));
    if (tot[ADJ_BZ] > 0) adj_blur_z_data<<<tot[ADJ_BZ], kThreads, 0, st>>>(c, vols, P(ADJ_BZ));
    if (tot[ADJ_TZ] > 0) adj_blurT_z<<<tot[ADJ_TZ], kThreads, 0, st>>>(c, vols, P(ADJ_TZ));
    if (tot[ADJ_TY] > 0) adj_blurT_y<<<tot[ADJ_TY], kThreads, 0, st>>>(c, vols, P(ADJ_TY));
    if (tot[ADJ_TX] > 0) adj_blurT_x_hbar<<<tot[ADJ_TX], kThreads, 0, st>>>(c, vols, P(ADJ_TX));
    if (tot[ADJ_NRM] > 0) adj_normals<<<tot[ADJ_NRM], kThreads, 0, st>>>(c, vols, P(ADJ_NRM));
    if (tot[ADJ_PT] > 0) adj_point<<<tot[ADJ_PT], b2, 0, st>>>(c, vols, P(ADJ_PT), grads);
    if (tot[ADJ_W] > 0) adj_w<<<tot[ADJ_W], b2, 0, st>>>(c, vols, P(ADJ_W));
    if (tot[ADJ_G] > 0) adj_gather<<<tot[ADJ_G], b2, 0, st>>>(c, vols, P(ADJ_G), flag);
    return cudaGetLastError();
}

}  // namespace rsf
