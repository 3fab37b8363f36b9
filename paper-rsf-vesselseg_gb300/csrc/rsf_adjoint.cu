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
// Kernels (one thread per voxel, grid-stride): blur recompute x, y, z (the z
// kernel also forms the data-term adjoint), transposed blur z, y, x (the x
// kernel forms H_bar), unit normals, the stencil adjoint with the pointwise
// terms and parameter sums, and the final D^T gather.  Scratch comes from the
// workspace pools; the layout is given in launch_step_adjoint.
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
template <class V>
__device__ __forceinline__ float dT_x(const AdjConst &c, long long j, long long N, V v) {
    float acc = 0.0f;
#pragma unroll
    for (int d = -1; d <= 1; d++) {
        const long long m = j + d;
        if (m < 0 || m >= N) continue;
        long long r, l;
        nb_x(c, m, (int)(m % c.W), r, l);
        const float coef = (r == j ? 0.5f : 0.0f) - (l == j ? 0.5f : 0.0f);
        if (coef != 0.0f) acc = fmaf(coef, v(m), acc);
    }
    return acc;
}
template <class V>
__device__ __forceinline__ float dT_axis(long long j, int q, int n, long long stride, V v) {
    float acc = 0.0f;
#pragma unroll
    for (int d = -1; d <= 1; d++) {
        const int qm = q + d;
        if (qm < 0 || qm >= n) continue;
        const long long m = j + (long long)d * stride;
        long long r, l;
        nb_axis(m, qm, n, stride, r, l);
        const float coef = (r == j ? 0.5f : 0.0f) - (l == j ? 0.5f : 0.0f);
        if (coef != 0.0f) acc = fmaf(coef, v(m), acc);
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

// Valid correlation along y: (Wv, H, L) -> (Wv, Hv, L), four fields.
__global__ void adj_blur_y(AdjConst c, const float *in, float *out) {
    const long long nin = (long long)c.Wv * c.H * c.L, n = (long long)c.Wv * c.Hv * c.L;
    for (long long o = grid_start(); o < n; o += grid_step()) {
        const int xv = (int)(o % c.Wv);
        const long long t1 = o / c.Wv;
        const int yv = (int)(t1 % c.Hv);
        const int z = (int)(t1 / c.Hv);
        const long long base = ((long long)z * c.H + yv) * c.Wv + xv;
        for (int f = 0; f < 4; f++) {
            float a = 0.0f;
            for (int t = 0; t < c.k; t++) a = fmaf(in[f * nin + base + (long long)t * c.Wv], c.taps[t], a);
            out[f * n + o] = a;
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
    for (long long o = grid_start(); o < n; o += grid_step()) {
        const int xv = (int)(o % c.Wv);
        const long long t1 = o / c.Wv;
        const int yv = (int)(t1 % c.Hv);
        const int zv = (int)(t1 / c.Hv);
        const long long base = (long long)zv * plane + (long long)yv * c.Wv + xv;
        float B[4];
        for (int f = 0; f < 4; f++) {
            float a = 0.0f;
            for (int t = 0; t < c.k; t++) a = fmaf(in[f * nin + base + (long long)t * plane], c.taps[t], a);
            B[f] = a;
        }
        const long long i = ((long long)(zv + c.r) * c.H + (yv + c.r)) * c.W + xv + c.r;
        const float I = img_at(img, i, c.img_f32);
        const float rb1 = __frcp_rn(B[1]), rb3 = __frcp_rn(B[3]);
        const float fo = B[0] * rb1, fi = B[2] * rb3;
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

// Transposed (full) correlation along z: (Wv, Hv, Lv) -> (Wv, Hv, L), two fields.
__global__ void adj_blurT_z(AdjConst c, const float *in, float *out) {
    const long long nin = (long long)c.Wv * c.Hv * c.Lv, n = (long long)c.Wv * c.Hv * c.L;
    const long long plane = (long long)c.Wv * c.Hv;
    for (long long o = grid_start(); o < n; o += grid_step()) {
        const long long p = o % plane;
        const int z = (int)(o / plane);
        const int t0 = max(0, z - c.Lv + 1), t1 = min(c.k - 1, z);
        for (int f = 0; f < 2; f++) {
            float a = 0.0f;
            for (int t = t0; t <= t1; t++) a = fmaf(in[f * nin + (long long)(z - t) * plane + p], c.taps[t], a);
            out[f * n + o] = a;
        }
    }
}

// Transposed correlation along y: (Wv, Hv, L) -> (Wv, H, L).
__global__ void adj_blurT_y(AdjConst c, const float *in, float *out) {
    const long long nin = (long long)c.Wv * c.Hv * c.L, n = (long long)c.Wv * c.H * c.L;
    for (long long o = grid_start(); o < n; o += grid_step()) {
        const int xv = (int)(o % c.Wv);
        const long long t1 = o / c.Wv;
        const int y = (int)(t1 % c.H);
        const int z = (int)(t1 / c.H);
        const int a0 = max(0, y - c.Hv + 1), a1 = min(c.k - 1, y);
        for (int f = 0; f < 2; f++) {
            float a = 0.0f;
            for (int t = a0; t <= a1; t++)
                a = fmaf(in[f * nin + ((long long)z * c.Hv + (y - t)) * c.Wv + xv], c.taps[t], a);
            out[f * n + o] = a;
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

// Unit normals n = g / (|g| + 1e-6).
__global__ void adj_normals(AdjConst c, const float *phi, float *nx, float *ny, float *nz) {
    const long long N = (long long)c.W * c.H * c.L;
    for (long long i = grid_start(); i < N; i += grid_step()) {
        const int x = (int)(i % c.W);
        const long long t1 = i / c.W;
        const int y = (int)(t1 % c.H);
        const int z = (int)(t1 / c.H);
        (void)x;
        const float gx = diff_x_at(c, phi, i), gy = diff_y_at(c, phi, i, y), gz = diff_z_at(c, phi, i, z);
        const float rs = __frcp_rn(sqrtf(gx * gx + gy * gy + gz * gz) + 1e-6f);
        nx[i] = gx * rs;
        ny[i] = gy * rs;
        nz[i] = gz * rs;
    }
}

// Stencil adjoint and pointwise terms: w_a = g_bar_a (to be gathered by D_a^T)
// and out = u + delta H_bar + delta' u dt (-data + nu kappa); parameter sums.
__global__ void adj_stencil(AdjConst c, const float *phi, const void *img, const float *u, const float *nx,
                            const float *ny, const float *nz, const float *hbar, const float *eo_v,
                            const float *ei_v, float *wx, float *wy, float *wz, float *out, double *grads) {
    const long long N = (long long)c.W * c.H * c.L;
    const long long plane = (long long)c.W * c.H;
    double s_l1 = 0.0, s_l2 = 0.0, s_mu = 0.0, s_nu = 0.0;
    auto kbar = [&](long long m) { return u[m] * c.dt * (c.nu * dirac_fast(phi[m], c.eps) - c.mu); };
    auto lbar = [&](long long m) { return u[m] * c.dt * c.mu; };
    for (long long i = grid_start(); i < N; i += grid_step()) {
        const int x = (int)(i % c.W);
        const long long t1 = i / c.W;
        const int y = (int)(t1 % c.H);
        const int z = (int)(t1 / c.H);
        const float ph = phi[i], ui = u[i];
        const float I = img_at(img, i, c.img_f32);
        const float delta = dirac_fast(ph, c.eps);
        const float ddelta = __fdividef(-2.0f * ph * delta, fmaf(ph, ph, c.eps * c.eps));
        long long rx, lx, ry, ly, rz, lz;
        nb_x(c, i, x, rx, lx);
        nb_axis(i, y, c.H, c.W, ry, ly);
        nb_axis(i, z, c.L, plane, rz, lz);
        const float gx = 0.5f * (phi[rx] - phi[lx]), gy = 0.5f * (phi[ry] - phi[ly]), gz = 0.5f * (phi[rz] - phi[lz]);
        const float mag = sqrtf(gx * gx + gy * gy + gz * gz);
        const float rs = __frcp_rn(mag + 1e-6f);
        const float inv_mag = mag > 0.0f ? __frcp_rn(mag) : 0.0f;
        const float kap = 0.5f * (nx[rx] - nx[lx]) + 0.5f * (ny[ry] - ny[ly]) + 0.5f * (nz[rz] - nz[lz]);
        const int yr = (int)((ry - i) / c.W) + y, yl = (int)((ly - i) / c.W) + y;
        const int zr = (int)((rz - i) / plane) + z, zl = (int)((lz - i) / plane) + z;
        const float lap = 0.5f * (diff_x_at(c, phi, rx) - diff_x_at(c, phi, lx)) +
                          0.5f * (diff_y_at(c, phi, ry, yr) - diff_y_at(c, phi, ly, yl)) +
                          0.5f * (diff_z_at(c, phi, rz, zr) - diff_z_at(c, phi, lz, zl));
        const float nbx = dT_x(c, i, N, kbar), nby = dT_axis(i, y, c.H, c.W, kbar),
                    nbz = dT_axis(i, z, c.L, plane, kbar);
        const float lbx = dT_x(c, i, N, lbar), lby = dT_axis(i, y, c.H, c.W, lbar),
                    lbz = dT_axis(i, z, c.L, plane, lbar);
        const float ndot = nbx * nx[i] + nby * ny[i] + nbz * nz[i];
        wx[i] = lbx + (nbx - ndot * gx * inv_mag) * rs;
        wy[i] = lby + (nby - ndot * gy * inv_mag) * rs;
        wz[i] = lbz + (nbz - ndot * gz * inv_mag) * rs;
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
        const double ud = (double)ui * (double)c.dt;
        s_l1 -= ud * (double)delta * (double)eo;
        s_l2 += ud * (double)delta * (double)ei;
        s_mu += ud * ((double)lap - (double)kap);
        s_nu += ud * (double)delta * (double)kap;
    }
    if (grads) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            s_l1 += __shfl_down_sync(0xffffffffu, s_l1, o);
            s_l2 += __shfl_down_sync(0xffffffffu, s_l2, o);
            s_mu += __shfl_down_sync(0xffffffffu, s_mu, o);
            s_nu += __shfl_down_sync(0xffffffffu, s_nu, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(grads + 0, s_l1);
            atomicAdd(grads + 1, s_l2);
            atomicAdd(grads + 2, s_mu);
            atomicAdd(grads + 3, s_nu);
        }
    }
}

// out += sum_a D_a^T w_a.
__global__ void adj_gather(AdjConst c, const float *wx, const float *wy, const float *wz, float *out) {
    const long long N = (long long)c.W * c.H * c.L;
    const long long plane = (long long)c.W * c.H;
    auto vx = [&](long long m) { return wx[m]; };
    auto vy = [&](long long m) { return wy[m]; };
    auto vz = [&](long long m) { return wz[m]; };
    for (long long i = grid_start(); i < N; i += grid_step()) {
        const long long t1 = i / c.W;
        const int y = (int)(t1 % c.H);
        const int z = (int)(t1 / c.H);
        out[i] += dT_x(c, i, N, vx) + dT_axis(i, y, c.H, c.W, vy) + dT_axis(i, z, c.L, plane, vz);
    }
}

unsigned blocks_for(long long n) {
    const long long b = (n + kThreads - 1) / kThreads;
    return (unsigned)(b < 152LL * 64 ? (b > 0 ? b : 1) : 152LL * 64);
}

}  // namespace

// Scratch (N = W H L; the pools hold 1, 4 and 4 N floats):
//   phi2 : H (blur input), later H_bar
//   xs   : blur-x fields (4 Wv H L), then [0, 2N) the valid-layout adjoint pair
//          and [2N, 4N) e_out, e_in; later w_x, w_y in [0, 2N)
//   ys   : blur-y fields (4 Wv Hv L), then the z-transposed pair [0, 2N), the
//          y-transposed pair at 2N; later the normals [0, 3N) and w_z at 3N
cudaError_t launch_step_adjoint(const float *taps, int k, float eps, float dt, float mu, float nu, float l1, float l2,
                                int boundary, int img_f32, const float *phi, const void *img, const float *u,
                                float *out, double *grads, int W, int H, int L, float *phi2, float *xs, float *ys,
                                cudaStream_t st) {
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
        adj_blur_y<<<blocks_for(ny), kThreads, 0, st>>>(c, xs, ys);
        adj_blur_z_data<<<blocks_for(nz), kThreads, 0, st>>>(c, ys, phi, img, u, xs, eo, ei);
        adj_blurT_z<<<blocks_for(ny), kThreads, 0, st>>>(c, xs, ys);
        adj_blurT_y<<<blocks_for(nx), kThreads, 0, st>>>(c, ys, ys + 2 * N);
        adj_blurT_x_hbar<<<blocks_for(N), kThreads, 0, st>>>(c, ys + 2 * N, img, hbar);
    } else {
        cudaError_t e = cudaMemsetAsync(hbar, 0, sizeof(float) * (size_t)N, st);
        if (e != cudaSuccess) return e;
    }
    float *nxb = ys, *nyb = ys + N, *nzb = ys + 2 * N;
    float *wx = xs, *wy = xs + N, *wz = ys + 3 * N;
    adj_normals<<<blocks_for(N), kThreads, 0, st>>>(c, phi, nxb, nyb, nzb);
    adj_stencil<<<blocks_for(N), kThreads, 0, st>>>(c, phi, img, u, nxb, nyb, nzb, hbar, eo, ei, wx, wy, wz, out,
                                                    grads);
    adj_gather<<<blocks_for(N), kThreads, 0, st>>>(c, wx, wy, wz, out);
    return cudaGetLastError();
}

}  // namespace rsf
