// rsf_adjoint.cu -- reverse-mode derivative of one RSF step.
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
// consecutive outputs per thread; the last three kernels run on 3-D grids,
// the others are grid-stride loops.  Scratch comes from the workspace pools;
// the layout is given in launch_step_adjoint.
#include <cuda_runtime.h>

#include "rsf_arith.cuh"
#include "rsf_internal.h"

namespace rsf {
namespace {

constexpr int kThreads = 256;

struct AdjConst {
    float taps[MAXK];
    int k, r;
    int W, H, L;
    int Wv, Hv, Lv;  // valid blur extents; all > 0 or all 0
    float eps, dt, mu, nu, l1, l2;
    int boundary;    // 0 reference (x = 0 reads the previous linear element), 1 clamp
    int img_f32;
};

__device__ __forceinline__ float img_at(const void *img, long long i, int f32) {
    return f32 ? static_cast<const float *>(img)[i] : (float)static_cast<const unsigned char *>(img)[i];
}

__device__ __forceinline__ long long grid_start() { return (long long)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ long long grid_step() { return (long long)gridDim.x * blockDim.x; }

// The stencil kernels run on 3-D grids of 32 x 8 blocks (x fastest, one z
// plane per blockIdx.z), so voxel coordinates need no 64-bit division.
constexpr int kBX = 32, kBY = 8;

// Right and left linear indices of the central difference at voxel i.
__device__ __forceinline__ void nb_x(const AdjConst &c, long long i, int x, long long &r, long long &l) {
    r = x + 1 < c.W ? i + 1 : i;
    if (x > 0) l = i - 1;
    else l = c.boundary == 0 ? (i > 0 ? i - 1 : 0) : i;
    if (x == c.W - 1) l = i - 1;
}
// y and z: (f[1] - f[0]) / 2 at 0, (f[n-1] - f[n-2]) / 2 at n - 1 (n >= 2).
__device__ __forceinline__ void nb_axis(long long i, int q, int n, long long stride, long long &r, long long &l) {
    const int qr = q + 1 < n ? q + 1 : n - 1;
    const int ql = q > 0 ? q - 1 : 0;
    r = i + (long long)(qr - q) * stride;
    l = i + (long long)(ql - q) * stride;
}

__device__ __forceinline__ float diff_x_at(const AdjConst &c, const float *f, long long m) {
    long long r, l;
    nb_x(c, m, (int)(m % c.W), r, l);
    return 0.5f * (f[r] - f[l]);
}
__device__ __forceinline__ float diff_y_at(const AdjConst &c, const float *f, long long m, int y) {
    long long r, l;
    nb_axis(m, y, c.H, c.W, r, l);
    return 0.5f * (f[r] - f[l]);
}
__device__ __forceinline__ float diff_z_at(const AdjConst &c, const float *f, long long m, int z) {
    long long r, l;
    nb_axis(m, z, c.L, (long long)c.W * c.H, r, l);
    return 0.5f * (f[r] - f[l]);
}

// (D_x^T v)(j): the neighbours j-1, j, j+1 in linear order are the only
// voxels whose difference reads j.
// x is j's x coordinate; the linear neighbours of a row's end are the next
// row's start and vice versa.  Branch-free: an out-of-range candidate is
// read as j itself with coefficient 0, so that all loads issue together.
template <class V>
__device__ __forceinline__ float dT_x(const AdjConst &c, long long j, int x, long long N, V v) {
    float acc = 0.0f;
#pragma unroll
    for (int d = -1; d <= 1; d++) {
        const long long m0 = j + d;
        const bool in = m0 >= 0 && m0 < N;
        const long long m = in ? m0 : j;
        const int mx = d == 0 ? x : d < 0 ? (x > 0 ? x - 1 : c.W - 1) : (x + 1 < c.W ? x + 1 : 0);
        long long r, l;
        nb_x(c, m, mx, r, l);
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

// delta(phi) with a fast division: the adjoint needs the derivative's value,
// not the forward's bit pattern.
__device__ __forceinline__ float dirac_fast(float phi, float eps) {
    return __fdividef(0.318309886183790672f * eps, fmaf(phi, phi, eps * eps));
}

__global__ void adj_heaviside(AdjConst c, const float *phi, float *h, long long N) {
    for (long long i = grid_start(); i < N; i += grid_step()) h[i] = heaviside<Arith::Portable>(phi[i], c.eps);
}

// Valid correlation along x of (I H, H, I (1-H), 1-H): (Wv, H, L) per field.
__global__ void adj_blur_x(AdjConst c, const float *h, const void *img, float *out) {
    const long long n = (long long)c.Wv * c.H * c.L;
    for (long long o = grid_start(); o < n; o += grid_step()) {
        const int xv = (int)(o % c.Wv);
        const long long row = o / c.Wv;  // z * H + y
        const long long base = row * c.W + xv;
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
        for (int t = 0; t < c.k; t++) {
            const float hv = h[base + t];
            const float I = img_at(img, base + t, c.img_f32);
            const float hi = 1.0f - hv;
            const float g = c.taps[t];
            a0 = fmaf(I * hv, g, a0);
            a1 = fmaf(hv, g, a1);
            a2 = fmaf(I * hi, g, a2);
            a3 = fmaf(hi, g, a3);
        }
        out[o] = a0;
        out[n + o] = a1;
        out[2 * n + o] = a2;
        out[3 * n + o] = a3;
    }
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

// Valid correlation along y: (Wv, H, L) -> (Wv, Hv, L), four fields.
__global__ void adj_blur_y(AdjConst c, const float *in, float *out) {
    const long long nin = (long long)c.Wv * c.H * c.L, n = (long long)c.Wv * c.Hv * c.L;
    const int nyb = (c.Hv + kNBy - 1) / kNBy;
    const long long cols = (long long)c.Wv * nyb * c.L;
    for (long long q = grid_start(); q < cols; q += grid_step()) {
        const int xv = (int)(q % c.Wv);
        const long long t1 = q / c.Wv;
        const int y0 = (int)(t1 % nyb) * kNBy;
        const int z = (int)(t1 / nyb);
        for (int f = 0; f < 4; f++) {
            float acc[kNBy];
            corr_block<kNBy, false>(c, in + f * nin + (long long)z * c.H * c.Wv + xv, c.Wv, y0, c.H, acc);
#pragma unroll
            for (int m = 0; m < kNBy; ++m)
                if (y0 + m < c.Hv) out[f * n + ((long long)z * c.Hv + y0 + m) * c.Wv + xv] = acc[m];
        }
    }
}

// Valid correlation along z, then the data-term adjoint at each valid voxel:
// writes (B1_bar - B3_bar, B2_bar - B4_bar) in the valid layout and e_out,
// e_in at the full-volume index.
__global__ void adj_blur_z_data(AdjConst c, const float *in, const float *phi, const void *img, const float *u,
                                float *pq, float *eo_out, float *ei_out) {
    const long long nin = (long long)c.Wv * c.Hv * c.L, n = (long long)c.Wv * c.Hv * c.Lv;
    const long long plane = (long long)c.Wv * c.Hv;
    const int nzb = (c.Lv + kNB - 1) / kNB;
    const long long cols = plane * nzb;
    for (long long q = grid_start(); q < cols; q += grid_step()) {
        const long long pxy = q % plane;
        const int z0 = (int)(q / plane) * kNB;
        const int xv = (int)(pxy % c.Wv), yv = (int)(pxy / c.Wv);
        float B[4][kNB];
        for (int f = 0; f < 4; f++) corr_block<kNB, false>(c, in + f * nin + pxy, plane, z0, c.L, B[f]);
#pragma unroll
        for (int m = 0; m < kNB; ++m) {
            const int zv = z0 + m;
            if (zv >= c.Lv) break;
            const long long o = (long long)zv * plane + pxy;
            const long long i = ((long long)(zv + c.r) * c.H + (yv + c.r)) * c.W + xv + c.r;
            const float I = img_at(img, i, c.img_f32);
            const float rb1 = __frcp_rn(B[1][m]), rb3 = __frcp_rn(B[3][m]);
            const float fo = B[0][m] * rb1, fi = B[2][m] * rb3;
            const float dfo = I - fo, dfi = I - fi;
            eo_out[i] = dfo * dfo;
            ei_out[i] = dfi * dfi;
            const float delta = dirac_fast(phi[i], c.eps);
            const float data_bar = -u[i] * c.dt * delta;
            const float fo_bar = -2.0f * dfo * (c.l1 * data_bar);
            const float fi_bar = -2.0f * dfi * (-c.l2 * data_bar);
            const float b1 = fo_bar * rb1, b2 = -fo_bar * fo * rb1;
            const float b3 = fi_bar * rb3, b4 = -fi_bar * fi * rb3;
            pq[o] = b1 - b3;
            pq[n + o] = b2 - b4;
        }
    }
}

// Transposed (full) correlation along z: (Wv, Hv, Lv) -> (Wv, Hv, L), two fields.
__global__ void adj_blurT_z(AdjConst c, const float *in, float *out) {
    const long long nin = (long long)c.Wv * c.Hv * c.Lv, n = (long long)c.Wv * c.Hv * c.L;
    const long long plane = (long long)c.Wv * c.Hv;
    const int nzb = (c.L + kNB - 1) / kNB;
    const long long cols = plane * nzb;
    for (long long q = grid_start(); q < cols; q += grid_step()) {
        const long long pxy = q % plane;
        const int z0 = (int)(q / plane) * kNB;
        for (int f = 0; f < 2; f++) {
            float acc[kNB];
            corr_block<kNB, true>(c, in + f * nin + pxy, plane, z0, c.Lv, acc);
#pragma unroll
            for (int m = 0; m < kNB; ++m)
                if (z0 + m < c.L) out[f * n + (long long)(z0 + m) * plane + pxy] = acc[m];
        }
    }
}

// Transposed correlation along y: (Wv, Hv, L) -> (Wv, H, L).
__global__ void adj_blurT_y(AdjConst c, const float *in, float *out) {
    const long long nin = (long long)c.Wv * c.Hv * c.L, n = (long long)c.Wv * c.H * c.L;
    const int nyb = (c.H + kNBy - 1) / kNBy;
    const long long cols = (long long)c.Wv * nyb * c.L;
    for (long long q = grid_start(); q < cols; q += grid_step()) {
        const int xv = (int)(q % c.Wv);
        const long long t1 = q / c.Wv;
        const int y0 = (int)(t1 % nyb) * kNBy;
        const int z = (int)(t1 / nyb);
        for (int f = 0; f < 2; f++) {
            float acc[kNBy];
            corr_block<kNBy, true>(c, in + f * nin + (long long)z * c.Hv * c.Wv + xv, c.Wv, y0, c.Hv, acc);
#pragma unroll
            for (int m = 0; m < kNBy; ++m)
                if (y0 + m < c.H) out[f * n + ((long long)z * c.H + y0 + m) * c.Wv + xv] = acc[m];
        }
    }
}

// Transposed correlation along x and H_bar = I * P~ + Q~ over the volume.
__global__ void adj_blurT_x_hbar(AdjConst c, const float *in, const void *img, float *hbar) {
    const long long nin = (long long)c.Wv * c.H * c.L, N = (long long)c.W * c.H * c.L;
    for (long long i = grid_start(); i < N; i += grid_step()) {
        const int x = (int)(i % c.W);
        const long long row = i / c.W;
        const int a0 = max(0, x - c.Wv + 1), a1 = min(c.k - 1, x);
        float p = 0.0f, q = 0.0f;
        for (int t = a0; t <= a1; t++) {
            const long long s = row * c.Wv + (x - t);
            p = fmaf(in[s], c.taps[t], p);
            q = fmaf(in[nin + s], c.taps[t], q);
        }
        hbar[i] = fmaf(img_at(img, i, c.img_f32), p, q);
    }
}

// Gradient g = D phi and unit normals n = g / (|g| + 1e-6), stored so that
// the stencil adjoint reads them at its neighbours instead of recomputing.
__global__ void adj_normals(AdjConst c, const float *phi, float *gxo, float *gyo, float *gzo, float *nx, float *ny,
                            float *nz) {
    const long long N = (long long)c.W * c.H * c.L;
    for (long long i = grid_start(); i < N; i += grid_step()) {
        const long long t1 = i / c.W;
        const int y = (int)(t1 % c.H);
        const int z = (int)(t1 / c.H);
        const float gx = diff_x_at(c, phi, i), gy = diff_y_at(c, phi, i, y), gz = diff_z_at(c, phi, i, z);
        const float rs = __frcp_rn(sqrtf(gx * gx + gy * gy + gz * gz) + 1e-6f);
        gxo[i] = gx;
        gyo[i] = gy;
        gzo[i] = gz;
        nx[i] = gx * rs;
        ny[i] = gy * rs;
        nz[i] = gz * rs;
    }
}

// Pointwise terms and parameter sums:
//   out = u + delta H_bar + delta' u dt (nu kappa - data),
// with kappa = sum_a D_a n_a and Lap = sum_a D_a g_a from the stored fields.
// A block covers a 32 x 8 column of kPointZ planes; the parameter sums are
// reduced in the block and added with one double atomic per parameter and
// block (the same four addresses for every block, so their number matters).
constexpr int kPointZ = 16;
__global__ void __launch_bounds__(kBX * kBY) adj_point(AdjConst c, const float *phi, const void *img,
                                                       const float *u, const float *gxa, const float *gya,
                                                       const float *gza, const float *nx, const float *ny,
                                                       const float *nz, const float *hbar, const float *eo_v,
                                                       const float *ei_v, float *out, double *grads) {
    const long long plane = (long long)c.W * c.H;
    float s_l1 = 0.0f, s_l2 = 0.0f, s_mu = 0.0f, s_nu = 0.0f;
    const int x = blockIdx.x * kBX + threadIdx.x, y = blockIdx.y * kBY + threadIdx.y;
    const int z0 = blockIdx.z * kPointZ, z1 = min(z0 + kPointZ, c.L);
    for (int z = z0; z < z1 && x < c.W && y < c.H; ++z) {
        const long long i = ((long long)z * c.H + y) * c.W + x;
        const float ph = phi[i], ui = u[i];
        const float I = img_at(img, i, c.img_f32);
        const float delta = dirac_fast(ph, c.eps);
        const float ddelta = __fdividef(-2.0f * ph * delta, fmaf(ph, ph, c.eps * c.eps));
        long long rx, lx, ry, ly, rz, lz;
        nb_x(c, i, x, rx, lx);
        nb_axis(i, y, c.H, c.W, ry, ly);
        nb_axis(i, z, c.L, plane, rz, lz);
        const float kap = 0.5f * (nx[rx] - nx[lx]) + 0.5f * (ny[ry] - ny[ly]) + 0.5f * (nz[rz] - nz[lz]);
        const float lap = 0.5f * (gxa[rx] - gxa[lx]) + 0.5f * (gya[ry] - gya[ly]) + 0.5f * (gza[rz] - gza[lz]);
        const bool valid = c.Wv > 0 && x >= c.r && x < c.r + c.Wv && y >= c.r && y < c.r + c.Hv && z >= c.r &&
                           z < c.r + c.Lv;
        float eo, ei;
        if (valid) {
            eo = eo_v[i];
            ei = ei_v[i];
        } else {  // border band: f_out = f_in = 30 / 30
            eo = ei = (I - 1.0f) * (I - 1.0f);
        }
        const float data = c.l1 * eo - c.l2 * ei;
        out[i] = ui + delta * hbar[i] + ddelta * ui * c.dt * (c.nu * kap - data);
        const float ud = ui * c.dt, udd = ud * delta;
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
// with n_bar = D^T kappa_bar, to be gathered by D_a^T.  Runs after adj_point,
// which has read H_bar, e_out and e_in: w is written over them.
__global__ void adj_w(AdjConst c, const float *phi, const float *u, const float *gxa, const float *gya,
                      const float *gza, const float *nx, const float *ny, const float *nz, float *wx, float *wy,
                      float *wz) {
    const long long N = (long long)c.W * c.H * c.L;
    const long long plane = (long long)c.W * c.H;
    auto kbar = [&](long long m) { return u[m] * c.dt * (c.nu * dirac_fast(phi[m], c.eps) - c.mu); };
    auto lbar = [&](long long m) { return u[m] * c.dt * c.mu; };
    const int x = blockIdx.x * kBX + threadIdx.x, y = blockIdx.y * kBY + threadIdx.y, z = blockIdx.z;
    if (x < c.W && y < c.H) {
        const long long i = ((long long)z * c.H + y) * c.W + x;
        const float gx = gxa[i], gy = gya[i], gz = gza[i];
        const float mag = sqrtf(gx * gx + gy * gy + gz * gz);
        const float rs = __frcp_rn(mag + 1e-6f);
        const float inv_mag = mag > 0.0f ? __frcp_rn(mag) : 0.0f;
        const float nbx = dT_x(c, i, x, N, kbar), nby = dT_axis(i, y, c.H, c.W, kbar),
                    nbz = dT_axis(i, z, c.L, plane, kbar);
        const float lbx = dT_x(c, i, x, N, lbar), lby = dT_axis(i, y, c.H, c.W, lbar),
                    lbz = dT_axis(i, z, c.L, plane, lbar);
        const float ndot = nbx * nx[i] + nby * ny[i] + nbz * nz[i];
        wx[i] = lbx + (nbx - ndot * gx * inv_mag) * rs;
        wy[i] = lby + (nby - ndot * gy * inv_mag) * rs;
        wz[i] = lbz + (nbz - ndot * gz * inv_mag) * rs;
    }
}

// out += sum_a D_a^T w_a; a non-finite result sets kFlagAdjointNonFinite.
__global__ void adj_gather(AdjConst c, const float *wx, const float *wy, const float *wz, float *out,
                           unsigned *flag) {
    const long long N = (long long)c.W * c.H * c.L;
    const long long plane = (long long)c.W * c.H;
    auto vx = [&](long long m) { return wx[m]; };
    auto vy = [&](long long m) { return wy[m]; };
    auto vz = [&](long long m) { return wz[m]; };
    const int x = blockIdx.x * kBX + threadIdx.x, y = blockIdx.y * kBY + threadIdx.y, z = blockIdx.z;
    if (x < c.W && y < c.H) {
        const long long i = ((long long)z * c.H + y) * c.W + x;
        const float v = out[i] + (dT_x(c, i, x, N, vx) + dT_axis(i, y, c.H, c.W, vy) + dT_axis(i, z, c.L, plane, vz));
        out[i] = v;
        if (!isfinite(v) && flag) atomicOr(flag, kFlagAdjointNonFinite);
    }
}

unsigned blocks_for(long long n) {
    const long long b = (n + kThreads - 1) / kThreads, cap = 64LL * sm_count();
    return (unsigned)(b < cap ? (b > 0 ? b : 1) : cap);
}

}  // namespace

// Scratch (N = W H L; the pools hold 1, 4 and 4 N floats):
//   phi2 : H (blur input), later H_bar, then w_x
//   xs   : blur-x fields (4 Wv H L), then [0, 2N) the valid-layout adjoint pair
//          and [2N, 4N) e_out, e_in (later w_y, w_z); then g_x, g_y in [0, 2N)
//   ys   : blur-y fields (4 Wv Hv L), then the z-transposed pair [0, 2N), the
//          y-transposed pair at 2N; later g_z, n_x, n_y, n_z
cudaError_t launch_step_adjoint(const float *taps, int k, float eps, float dt, float mu, float nu, float l1, float l2,
                                int boundary, int img_f32, const float *phi, const void *img, const float *u,
                                float *out, double *grads, int W, int H, int L, float *phi2, float *xs, float *ys,
                                unsigned *flag, cudaStream_t st) {
    AdjConst c;
    for (int t = 0; t < MAXK; t++) c.taps[t] = t < k ? taps[t] : 0.0f;
    c.k = k;
    c.r = (k - 1) / 2;
    c.W = W;
    c.H = H;
    c.L = L;
    c.Wv = W - k + 1;
    c.Hv = H - k + 1;
    c.Lv = L - k + 1;
    if (c.Wv <= 0 || c.Hv <= 0 || c.Lv <= 0) c.Wv = c.Hv = c.Lv = 0;
    c.eps = eps;
    c.dt = dt;
    c.mu = mu;
    c.nu = nu;
    c.l1 = l1;
    c.l2 = l2;
    c.boundary = boundary;
    c.img_f32 = img_f32;
    const long long N = (long long)W * H * L;
    float *hbar = phi2;
    float *eo = xs + 2 * N, *ei = xs + 3 * N;
    if (c.Wv > 0) {
        const long long nx = (long long)c.Wv * H * L, ny = (long long)c.Wv * c.Hv * L;
        const long long nz = (long long)c.Wv * c.Hv * c.Lv;
        adj_heaviside<<<blocks_for(N), kThreads, 0, st>>>(c, phi, phi2, N);
        adj_blur_x<<<blocks_for(nx), kThreads, 0, st>>>(c, phi2, img, xs);
        const long long pl = (long long)c.Wv * c.Hv;
        adj_blur_y<<<blocks_for((long long)c.Wv * L * ((c.Hv + kNBy - 1) / kNBy)), kThreads, 0, st>>>(c, xs, ys);
        adj_blur_z_data<<<blocks_for(pl * ((c.Lv + kNB - 1) / kNB)), kThreads, 0, st>>>(c, ys, phi, img, u, xs,
                                                                                          eo, ei);
        adj_blurT_z<<<blocks_for(pl * ((L + kNB - 1) / kNB)), kThreads, 0, st>>>(c, xs, ys);
        adj_blurT_y<<<blocks_for((long long)c.Wv * L * ((H + kNBy - 1) / kNBy)), kThreads, 0, st>>>(c, ys,
                                                                                                 ys + 2 * N);
        adj_blurT_x_hbar<<<blocks_for(N), kThreads, 0, st>>>(c, ys + 2 * N, img, hbar);
    } else {
        cudaError_t e = cudaMemsetAsync(hbar, 0, sizeof(float) * (size_t)N, st);
        if (e != cudaSuccess) return e;
    }
    float *gxb = xs, *gyb = xs + N, *gzb = ys, *nxb = ys + N, *nyb = ys + 2 * N, *nzb = ys + 3 * N;
    adj_normals<<<blocks_for(N), kThreads, 0, st>>>(c, phi, gxb, gyb, gzb, nxb, nyb, nzb);
    const dim3 g3((unsigned)((W + kBX - 1) / kBX), (unsigned)((H + kBY - 1) / kBY), (unsigned)L), b3(kBX, kBY, 1);
    const dim3 gp((unsigned)((W + kBX - 1) / kBX), (unsigned)((H + kBY - 1) / kBY),
                  (unsigned)((L + kPointZ - 1) / kPointZ));
    adj_point<<<gp, b3, 0, st>>>(c, phi, img, u, gxb, gyb, gzb, nxb, nyb, nzb, hbar, eo, ei, out, grads);
    adj_w<<<g3, b3, 0, st>>>(c, phi, u, gxb, gyb, gzb, nxb, nyb, nzb, hbar, eo, ei);
    adj_gather<<<g3, b3, 0, st>>>(c, hbar, eo, ei, out, flag);
    return cudaGetLastError();
}

}  // namespace rsf
