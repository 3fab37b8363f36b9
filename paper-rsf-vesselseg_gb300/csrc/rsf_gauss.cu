// rsf_gauss.cu -- the expanded Gaussian data term (rsf_params.data_term =
// RSF_DATA_TERM_GAUSSIAN; this project's own opt-in mode: the reference's
// kernel.cu:25-55 takes e = (I - f)^2 at the voxel).  It is the
// region-scalable fitting energy's data term written out,
//   e_i(c) = I(c)^2 (K*1)(c) - 2 I(c) (K*f_i)(c) + (K*f_i^2)(c),
// on the valid region of the blur, where K is the same valid separable
// correlation as the local fits (x, then y, then z, taps ascending, fused
// multiply-adds from +0) and f_i the full-volume fit field (1 in the border
// band, as 30/30).  K*1 is the constant s3 of every valid voxel.  In FP32:
//   b = fma(I*I, s3, K*f^2);  e = fma(-2 I, K*f, b).
// The border band keeps e = (I - 1)^2.  Kernels, after a z-pass that stored
// f_out, f_in of the valid region (the run-time-k path):
//   gauss_x      f_out, f_out^2, f_in, f_in^2 correlated along x (scratch G)
//   (y)          ypass_generic_kernel<1> correlates G along y into yb
//   gauss_z      along z, then e_out, e_in and lambda (e_out - e_in)
//   gauss_border lambda (e_out - e_in) of the border band
// All four write the data factor of every voxel after the fits, as the box
// e-term does, and the stencil reads it from there.
#include "rsf_kernels.cuh"

namespace rsf {
namespace {

// f_out, f_in at voxel (x, y, z): the z-pass's fits inside the valid region,
// 1 in the border band.
__device__ __forceinline__ float2 fits_at(const SubVolDev &s, int r, int x, int y, int z) {
    const int xv = x - r, yv = y - r, zv = z - r;
    if (s.Wv > 0 && (unsigned)xv < (unsigned)s.Wv && (unsigned)yv < (unsigned)s.Hv && (unsigned)zv < (unsigned)s.Lv) {
        const size_t di = ((size_t)zv * s.Hv + yv) * s.Wp + xv;
        return make_float2(__ldg(s.db + di), __ldg(s.db + (size_t)s.Wp * s.Hv * s.Lv + di));
    }
    return make_float2(1.0f, 1.0f);
}

__global__ void __launch_bounds__(GX_T) gauss_x_kernel(const SubVolDev *__restrict__ svs,
                                                       const int *__restrict__ pre, const StepConst c) {
    __shared__ float taps_s[MAXK];
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int ntx = (s.Wv + GX_T * GX_NB - 1) / (GX_T * GX_NB);
    const int tx = t % ntx;
    t /= ntx;
    const int y = t % s.H, z = t / s.H;
    for (int i = threadIdx.x; i < c.k; i += blockDim.x) taps_s[i] = c.taps[i];
    __syncthreads();
    const int x0 = (tx * GX_T + threadIdx.x) * GX_NB;
    if (x0 >= s.Wv) return;
    float acc[4][GX_NB];
#pragma unroll
    for (int f = 0; f < 4; ++f)
#pragma unroll
        for (int m = 0; m < GX_NB; ++m) acc[f][m] = 0.0f;
    for (int q = 0; q < GX_NB + c.k - 1; ++q) {
        const int x = x0 + q;
        float v[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // inputs past W feed only outputs past Wv
        if (x < s.W) {
            const float2 f = fits_at(s, c.r, x, y, z);
            v[0] = f.x;
            v[1] = __fmul_rn(f.x, f.x);
            v[2] = f.y;
            v[3] = __fmul_rn(f.y, f.y);
        }
#pragma unroll
        for (int m = 0; m < GX_NB; ++m) {
            const int tt = q - m;
            if (tt >= 0 && tt < c.k)
#pragma unroll
                for (int f = 0; f < 4; ++f) acc[f][m] = __fmaf_rn(v[f], taps_s[tt], acc[f][m]);
        }
    }
    float *g = s.xb + c.gdelta + ((size_t)z * s.H + y) * s.Wp + x0;
    const size_t fs = (size_t)s.Wp * s.H * s.L;
#pragma unroll
    for (int f = 0; f < 4; ++f)
#pragma unroll
        for (int m = 0; m < GX_NB; ++m)
            if (x0 + m < s.Wv) g[f * fs + m] = acc[f][m];
}

template <bool DEBUG>
__global__ void __launch_bounds__(ZB_TX) gauss_z_kernel(const SubVolDev *__restrict__ svs,
                                                        const int *__restrict__ pre, const StepConst c, DebugOut dbg) {
    __shared__ float taps_s[MAXK];
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int ntx = (s.Wv + ZB_TX - 1) / ZB_TX, ntz = (s.Lv + ZB_ZB - 1) / ZB_ZB;
    const int tx = t % ntx;
    t /= ntx;
    const int tz = t % ntz;
    const int y = t / ntz;
    for (int i = threadIdx.x; i < c.k; i += blockDim.x) taps_s[i] = c.taps[i];
    __syncthreads();
    const int x = tx * ZB_TX + threadIdx.x;
    if (x >= s.Wv) return;
    const int z0 = tz * ZB_ZB;
    const size_t fs = (size_t)s.Wp * s.Hv * s.L, ps = (size_t)s.Wp * s.Hv;
    const float *col = s.yb + (size_t)y * s.Wp + x;
    float kf_o[ZB_ZB], kff_o[ZB_ZB], kf_i[ZB_ZB], kff_i[ZB_ZB];
    conv_block_rt<ZB_ZB>(col, ps, z0, s.L, taps_s, c.k, kf_o);
    conv_block_rt<ZB_ZB>(col + fs, ps, z0, s.L, taps_s, c.k, kff_o);
    conv_block_rt<ZB_ZB>(col + 2 * fs, ps, z0, s.L, taps_s, c.k, kf_i);
    conv_block_rt<ZB_ZB>(col + 3 * fs, ps, z0, s.L, taps_s, c.k, kff_i);
    const int r = c.r;
    float *dfull = s.db + 2 * (size_t)s.Wp * s.Hv * s.Lv;
#pragma unroll
    for (int m = 0; m < ZB_ZB; ++m) {
        const int o = z0 + m;
        if (o >= s.Lv) break;
        const size_t vi = ((size_t)(o + r) * s.H + (y + r)) * s.W + (x + r);
        const float I = load_img(s.img, vi, c.img_f32);
        const float a = __fmul_rn(I, I), m2 = __fmul_rn(-2.0f, I);
        const float eo = __fmaf_rn(m2, kf_o[m], __fmaf_rn(a, c.s3, kff_o[m]));
        const float ei = __fmaf_rn(m2, kf_i[m], __fmaf_rn(a, c.s3, kff_i[m]));
        dfull[vi] = data_factor(eo, ei, c.l1, c.l2, c.lam_equal != 0);
        if (DEBUG) {
            dbg.f[2 * dbg.n + vi] = eo;
            dbg.f[3 * dbg.n + vi] = ei;
        }
    }
}

template <bool DEBUG>
__global__ void __launch_bounds__(GB_T) gauss_border_kernel(const SubVolDev *__restrict__ svs,
                                                            const int *__restrict__ pre, const StepConst c,
                                                            DebugOut dbg) {
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    const long long i = (long long)(b - __ldg(pre + sv)) * GB_T + threadIdx.x;
    const long long WH = (long long)s.W * s.H;
    if (i >= WH * s.L) return;
    const int z = (int)(i / WH), rem = (int)(i - (long long)z * WH), y = rem / s.W, x = rem - y * s.W;
    const int r = c.r;
    const bool inside = s.Wv > 0 && (unsigned)(x - r) < (unsigned)s.Wv && (unsigned)(y - r) < (unsigned)s.Hv &&
                        (unsigned)(z - r) < (unsigned)s.Lv;
    if (inside) return;
    const float I = load_img(s.img, (size_t)i, c.img_f32);
    const float d = __fsub_rn(I, 1.0f);
    const float e = __fmul_rn(d, d);
    s.db[2 * (size_t)s.Wp * s.Hv * s.Lv + (size_t)i] = data_factor(e, e, c.l1, c.l2, c.lam_equal != 0);
    if (DEBUG) {
        dbg.f[2 * dbg.n + i] = e;
        dbg.f[3 * dbg.n + i] = e;
    }
}

}  // namespace

cudaError_t launch_gauss(const SubVolDev *svs, const int *pre, int n1, const int *tot, const StepConst &c,
                         const DebugOut *dbg, cudaStream_t st) {
    const DebugOut none = {nullptr, 0};
    if (tot[NKERN] > 0) gauss_x_kernel<<<tot[NKERN], GX_T, 0, st>>>(svs, pre + NKERN * n1, c);
    if (tot[NKERN + 1] > 0) ypass_generic_kernel<1><<<tot[NKERN + 1], YB_TX, 0, st>>>(svs, pre + (NKERN + 1) * n1, c);
    if (tot[NKERN + 2] > 0) {
        if (dbg) gauss_z_kernel<true><<<tot[NKERN + 2], ZB_TX, 0, st>>>(svs, pre + (NKERN + 2) * n1, c, *dbg);
        else gauss_z_kernel<false><<<tot[NKERN + 2], ZB_TX, 0, st>>>(svs, pre + (NKERN + 2) * n1, c, none);
    }
    if (tot[NKERN + 3] > 0) {
        if (dbg) gauss_border_kernel<true><<<tot[NKERN + 3], GB_T, 0, st>>>(svs, pre + (NKERN + 3) * n1, c, *dbg);
        else gauss_border_kernel<false><<<tot[NKERN + 3], GB_T, 0, st>>>(svs, pre + (NKERN + 3) * n1, c, none);
    }
    return cudaGetLastError();
}

}  // namespace rsf
