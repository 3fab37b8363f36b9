// rsf_kernels.cuh -- device code of one RSF iteration: four kernels per step.
//
//   x-pass   phi, I -> H, 1-H, I*H, I*(1-H) (kernel.cu:210-298) and their
//            valid correlation along x (kernel.cu:1000-1014)
//   y-pass   valid correlation along y (kernel.cu:1017-1031)
//   z-pass   valid correlation along z (kernel.cu:1035-1049), local fits
//            f = blur(I H)/blur(H) (kernel.cu:191-207), e = (I - f)^2
//            (kernel.cu:25-55) and the data factor lambda (e_out - e_in)
//   stencil  gradient, |gradient|, normalised gradient, curvature and the
//            "Laplacian" with the reference's boundary rules (kernel.cu:57-125,
//            173-189, 630-933), the border band f = 30/30 (kernel.cu:300-325),
//            delta (kernel.cu:265-280) and the explicit update
//            (kernel.cu:365-387); writes phi once.
//
// Every kernel takes the whole batch: a table of sub-volumes and, per kernel,
// a prefix sum of the blocks each sub-volume needs (block b finds its
// sub-volume by binary search).  A single volume is a batch of one.
//
// Summation order is the reference's: each blurred value is accumulated with
// fused multiply-adds from +0 over ascending taps, x first, then y, then z.
// The y and z correlations stream along their axis with K rotating
// accumulators per column (the accumulator of output o is slot o mod K), so
// every input is loaded once; two adjacent columns share one thread and one
// packed f32x2 multiply-add, which rounds each lane exactly like fmaf.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "rsf_arith.cuh"
#include "rsf_internal.h"

#ifndef RSF_F32X2
#define RSF_F32X2 1
#endif

namespace rsf {

enum { F_H = 0, F_HI = 1, F_IH = 2, F_IHI = 3 };  // field order in the x/y buffers

__device__ __forceinline__ int find_sv(const int *__restrict__ pre, int n, int b) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(pre + mid) <= b) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ float load_img(const void *img, size_t i, int f32) {
    return f32 ? __ldg(static_cast<const float *>(img) + i)
               : (float)__ldg(static_cast<const unsigned char *>(img) + i);
}

// d = a * b + c on both lanes, each rounded once (IEEE fma).
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
#if RSF_F32X2
    unsigned long long ua, ub, uc, ud;
    asm("mov.b64 %0, {%1, %2};" : "=l"(ua) : "f"(a.x), "f"(a.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(ub) : "f"(b.x), "f"(b.y));
    asm("mov.b64 %0, {%1, %2};" : "=l"(uc) : "f"(c.x), "f"(c.y));
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(ud) : "l"(ua), "l"(ub), "l"(uc));
    float2 d;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(ud));
    return d;
#else
    return make_float2(__fmaf_rn(a.x, b.x, c.x), __fmaf_rn(a.y, b.y, c.y));
#endif
}

__device__ __forceinline__ float2 ld2(const float *p) { return __ldg(reinterpret_cast<const float2 *>(p)); }

// Valid correlation of XB consecutive outputs of one packed field pair:
// src points at the lane's first input, consecutive inputs are two float2
// apart (the shared slab holds float4 (H, 1-H, I H, I (1-H)) per element).
template <int K, int XB>
__device__ __forceinline__ void xconv_pair(const float2 *src, const StepConst &c, const float2 *taps_s, int k,
                                           float2 (&acc)[XB]) {
    if constexpr (K > 0) {
#pragma unroll
        for (int q = 0; q < XB + K - 1; ++q) {
            const float2 v = src[2 * q];
#pragma unroll
            for (int m = 0; m < XB; ++m) {
                const int tt = q - m;
                if (tt == 0) acc[m] = fma2(v, c.taps2[0], make_float2(0.f, 0.f));
                else if (tt > 0 && tt < K) acc[m] = fma2(v, c.taps2[tt], acc[m]);
            }
        }
    } else {
#pragma unroll
        for (int m = 0; m < XB; ++m) acc[m] = make_float2(0.f, 0.f);
        for (int q = 0; q < XB + k - 1; ++q) {
            const float2 v = src[2 * q];
#pragma unroll
            for (int m = 0; m < XB; ++m) {
                const int tt = q - m;
                if (tt >= 0 && tt < k) acc[m] = fma2(v, taps_s[tt], acc[m]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// x-pass.  One warp per row segment of 32*XB outputs.  The four fields of
// the segment's inputs sit in shared memory as float4 (H, 1-H, I H, I (1-H));
// a lane produces XB consecutive outputs of one packed field pair at a time
// (XB odd, so the lanes' 64-bit loads fall in distinct banks), the results
// are staged in shared memory and written as float4 rows.
// Shared memory: XP_ROWS * span float4 inputs, MAXK float2 taps (generic k),
// XP_ROWS * 2 * XT floats of pair-0 staging.
// ---------------------------------------------------------------------------
template <int K, int XB, Arith A>
__global__ void __launch_bounds__(XP_ROWS * 32) xpass_kernel(const SubVolDev *__restrict__ svs,
                                                              const int *__restrict__ pre,
                                                              const StepConst c, int parity) {
    extern __shared__ float4 sm4[];
    constexpr int XT = 32 * XB;
    const int k = K > 0 ? K : c.k;
    const int span = XT + k - 1;
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int ntx = (s.Wv + XT - 1) / XT, nty = (s.H + XP_ROWS - 1) / XP_ROWS;
    const int tx = t % ntx;
    t /= ntx;
    const int ty = t % nty;
    const int z = t / nty;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y = ty * XP_ROWS + warp;
    float2 *taps_s = reinterpret_cast<float2 *>(sm4 + XP_ROWS * span);  // MAXK pairs, then the pair-0 stages
    if (K == 0) {
        for (int i = threadIdx.x; i < k; i += blockDim.x) taps_s[i] = c.taps2[i];
        __syncthreads();
    }
    if (y >= s.H) return;
    float4 *in = sm4 + warp * span;
    const int x0 = tx * XT;
    const size_t row = ((size_t)z * s.H + y) * s.W;
    const float *phi = (parity ? s.phi[1] : s.phi[0]) + row;
    for (int e = lane; e < span; e += 32) {
        const int x = x0 + e;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (x < s.W) {
            const float h = heaviside<A>(__ldg(phi + x), c.eps);
            const float I = load_img(s.img, row + x, c.img_f32);
            const float hi = __fsub_rn(1.0f, h);
            v = make_float4(h, hi, __fmul_rn(I, h), __fmul_rn(I, hi));
        }
        in[e] = v;
    }
    __syncwarp();
    // Pair 0 (H, 1-H) is staged in its own slab, pair 1 (I H, I (1-H)) in
    // the input slab once every lane has finished reading it.
    float *st01 = reinterpret_cast<float *>(sm4 + XP_ROWS * span) + 2 * MAXK + warp * 2 * XT;
    float *st23 = reinterpret_cast<float *>(in);
    const float2 *src = reinterpret_cast<const float2 *>(in + XB * lane);
    float2 acc[XB];
    xconv_pair<K, XB>(src, c, taps_s, k, acc);
#pragma unroll
    for (int m = 0; m < XB; ++m) {
        st01[XB * lane + m] = acc[m].x;
        st01[XT + XB * lane + m] = acc[m].y;
    }
    xconv_pair<K, XB>(src + 1, c, taps_s, k, acc);
    __syncwarp();
#pragma unroll
    for (int m = 0; m < XB; ++m) {
        st23[XB * lane + m] = acc[m].x;
        st23[XT + XB * lane + m] = acc[m].y;
    }
    __syncwarp();
    const size_t fstride = (size_t)s.Wp * s.H * s.L;
    const size_t orow = ((size_t)z * s.H + y) * s.Wp;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
        const float4 *sf = reinterpret_cast<const float4 *>((f < 2 ? st01 : st23) + (f & 1) * XT);
        float4 *dst = reinterpret_cast<float4 *>(s.xb + f * fstride + orow + x0);
        for (int e = lane; e < XT / 4; e += 32)
            if (x0 + 4 * e < s.Wv) dst[e] = sf[e];
    }
}

// ---------------------------------------------------------------------------
// Streaming valid correlation along a strided axis for a pair of columns:
// inputs src[i * stride] for i in [0, n), outputs o = i - K + 1 in [0, n-K+1)
// handed to emit(o, value) as soon as they complete.
// ---------------------------------------------------------------------------
template <int K, bool GUARD, typename Emit>
__device__ __forceinline__ void stream_block(const float *src, size_t stride, int base, int n, const StepConst &c,
                                             float2 (&acc)[K], Emit &emit) {
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const int i = base + j;
        if (GUARD && i >= n) break;
        const float2 v = ld2(src + (size_t)i * stride);
#pragma unroll
        for (int tt = 0; tt < K; ++tt) {
            const int slot = (j - tt + K) % K;
            if (tt == 0) acc[slot] = fma2(v, c.taps2[0], make_float2(0.f, 0.f));
            else acc[slot] = fma2(v, c.taps2[tt], acc[slot]);
        }
        const int o = i - (K - 1);
        if (o >= 0) emit(o, acc[(j + 1) % K]);
    }
}

template <int K, typename Emit>
__device__ __forceinline__ void stream_axis(const float *src, size_t stride, int n, const StepConst &c, Emit &emit) {
    float2 acc[K];
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] = make_float2(0.f, 0.f);
    int base = 0;
    for (; base + K <= n; base += K) stream_block<K, false>(src, stride, base, n, c, acc, emit);
    if (base < n) stream_block<K, true>(src, stride, base, n, c, acc, emit);
}

// Register-blocked version for a tap count known only at run time: NB
// consecutive outputs per call, same accumulation order.
template <int NB>
__device__ __forceinline__ void conv_block_rt(const float *__restrict__ base, size_t stride, int start, int n,
                                              const float *taps_s, int k, float (&acc)[NB]) {
#pragma unroll
    for (int m = 0; m < NB; ++m) acc[m] = 0.0f;
    for (int q = 0; q < NB + k - 1; ++q) {
        const int p = start + q;
        const float v = (p >= 0 && p < n) ? __ldg(base + (size_t)p * stride) : 0.0f;
#pragma unroll
        for (int m = 0; m < NB; ++m) {
            const int tt = q - m;
            if (tt >= 0 && tt < k) acc[m] = __fmaf_rn(v, taps_s[tt], acc[m]);
        }
    }
}

// ---------------------------------------------------------------------------
// y-pass.  One thread streams a column pair of one field of one z plane.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(YP_PAIRS) ypass_kernel(const SubVolDev *__restrict__ svs,
                                                         const int *__restrict__ pre, const StepConst c) {
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int ntx = (s.Wv + 2 * YP_PAIRS - 1) / (2 * YP_PAIRS);
    const int tx = t % ntx;
    t /= ntx;
    const int f = t & 3;
    const int z = t >> 2;
    const int x = 2 * (tx * YP_PAIRS + threadIdx.x);
    if (x >= s.Wv) return;
    const float *src = s.xb + f * ((size_t)s.Wp * s.H * s.L) + (size_t)z * s.H * s.Wp + x;
    float *dst = s.yb + f * ((size_t)s.Wp * s.Hv * s.L) + (size_t)z * s.Hv * s.Wp + x;
    const size_t wp = (size_t)s.Wp;
    auto emit = [&](int o, float2 v) { *reinterpret_cast<float2 *>(dst + (size_t)o * wp) = v; };
    stream_axis<K>(src, wp, s.H, c, emit);
}

template <int U = 0>
__global__ void __launch_bounds__(YB_TX) ypass_generic_kernel(const SubVolDev *__restrict__ svs,
                                                              const int *__restrict__ pre, const StepConst c) {
    __shared__ float taps_s[MAXK];
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int ntx = (s.Wv + YB_TX - 1) / YB_TX, nty = (s.Hv + YB_YB - 1) / YB_YB;
    const int tx = t % ntx;
    t /= ntx;
    const int ty = t % nty;
    t /= nty;
    const int f = t & 3;
    const int z = t >> 2;
    for (int i = threadIdx.x; i < c.k; i += blockDim.x) taps_s[i] = c.taps[i];
    __syncthreads();
    const int x = tx * YB_TX + threadIdx.x;
    if (x >= s.Wv) return;
    const int y0 = ty * YB_YB;
    const float *src = s.xb + f * ((size_t)s.Wp * s.H * s.L) + (size_t)z * s.H * s.Wp + x;
    float *dst = s.yb + f * ((size_t)s.Wp * s.Hv * s.L) + (size_t)z * s.Hv * s.Wp + x;
    float acc[YB_YB];
    conv_block_rt<YB_YB>(src, (size_t)s.Wp, y0, s.H, taps_s, c.k, acc);
#pragma unroll
    for (int m = 0; m < YB_YB; ++m)
        if (y0 + m < s.Hv) dst[(size_t)(y0 + m) * s.Wp] = acc[m];
}

// ---------------------------------------------------------------------------
// z-pass.  Four lanes per column pair, one field each, streaming z.  When an
// output plane completes, the lanes exchange their blurred values so that
// each lane forms one local fit (f_out or f_in of one of the two columns) and
// its e term; lanes 0 and 2 of the group write lambda (e_out - e_in).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void fits_and_data(const SubVolDev &s, const StepConst &c, int f, int x, int y, int o,
                                              bool act, float2 B, const DebugOut &dbg, bool debug) {
    // lane f: 0 -> f_out(x), 1 -> f_in(x), 2 -> f_out(x+1), 3 -> f_in(x+1)
    const float bx_hi = __shfl_down_sync(0xffffffffu, B.x, 2);  // lanes 0,1 get IH(x), IHI(x)
    const float by_lo = __shfl_up_sync(0xffffffffu, B.y, 2);    // lanes 2,3 get H(x+1), HI(x+1)
    const float num = f < 2 ? bx_hi : B.y;
    const float den = f < 2 ? B.x : by_lo;
    const float fv = __fdiv_rn(num, den);
    const int xc = x + (f >> 1);
    const int r = c.r;
    float I = 0.0f;
    const size_t vi = ((size_t)(o + r) * s.H + (y + r)) * s.W + (xc + r);
    const bool live = act && xc < s.Wv;
    if (live) I = load_img(s.img, vi, c.img_f32);
    const float d = __fsub_rn(I, fv);
    const float e = __fmul_rn(d, d);
    const float e_in = __shfl_down_sync(0xffffffffu, e, 1);  // lanes 0, 2 get e_in of their column
    if (live && (f & 1) == 0)
        s.db[((size_t)o * s.Hv + y) * s.Wp + xc] = data_factor(e, e_in, c.l1, c.l2, c.lam_equal != 0);
    if (debug && live) {
        dbg.f[(size_t)(f & 1) * dbg.n + vi] = fv;
        dbg.f[(size_t)(2 + (f & 1)) * dbg.n + vi] = e;
    }
}

template <int K, bool DEBUG>
__global__ void __launch_bounds__(ZP_PAIRS * 4) zpass_kernel(const SubVolDev *__restrict__ svs,
                                                             const int *__restrict__ pre, const StepConst c,
                                                             DebugOut dbg) {
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int ntx = (s.Wv + 2 * ZP_PAIRS - 1) / (2 * ZP_PAIRS);
    const int tx = t % ntx;
    const int y = t / ntx;
    const int f = threadIdx.x & 3;
    const int x = 2 * (tx * ZP_PAIRS + (threadIdx.x >> 2));
    const bool act = x < s.Wv;
    const float *src = s.yb + f * ((size_t)s.Wp * s.Hv * s.L) + (size_t)y * s.Wp + (act ? x : 0);
    const size_t pstride = (size_t)s.Wp * s.Hv;
    auto emit = [&](int o, float2 v) { fits_and_data(s, c, f, x, y, o, act, v, dbg, DEBUG); };
    stream_axis<K>(src, pstride, s.L, c, emit);
}

template <bool DEBUG>
__global__ void __launch_bounds__(ZB_TX) zpass_generic_kernel(const SubVolDev *__restrict__ svs,
                                                              const int *__restrict__ pre, const StepConst c,
                                                              DebugOut dbg) {
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
    float num[ZB_ZB], den[ZB_ZB], fo[ZB_ZB], fi[ZB_ZB];
    conv_block_rt<ZB_ZB>(col + F_IH * fs, ps, z0, s.L, taps_s, c.k, num);
    conv_block_rt<ZB_ZB>(col + F_H * fs, ps, z0, s.L, taps_s, c.k, den);
#pragma unroll
    for (int m = 0; m < ZB_ZB; ++m) fo[m] = __fdiv_rn(num[m], den[m]);
    conv_block_rt<ZB_ZB>(col + F_IHI * fs, ps, z0, s.L, taps_s, c.k, num);
    conv_block_rt<ZB_ZB>(col + F_HI * fs, ps, z0, s.L, taps_s, c.k, den);
#pragma unroll
    for (int m = 0; m < ZB_ZB; ++m) fi[m] = __fdiv_rn(num[m], den[m]);
    const int r = c.r;
#pragma unroll
    for (int m = 0; m < ZB_ZB; ++m) {
        const int o = z0 + m;
        if (o >= s.Lv) break;
        const size_t vi = ((size_t)(o + r) * s.H + (y + r)) * s.W + (x + r);
        const float I = load_img(s.img, vi, c.img_f32);
        const float d_o = __fsub_rn(I, fo[m]), d_i = __fsub_rn(I, fi[m]);
        const float eo = __fmul_rn(d_o, d_o), ei = __fmul_rn(d_i, d_i);
        s.db[((size_t)o * s.Hv + y) * s.Wp + x] = data_factor(eo, ei, c.l1, c.l2, c.lam_equal != 0);
        if (DEBUG) {
            dbg.f[0 * dbg.n + vi] = fo[m];
            dbg.f[1 * dbg.n + vi] = fi[m];
            dbg.f[2 * dbg.n + vi] = eo;
            dbg.f[3 * dbg.n + vi] = ei;
        }
    }
}

// ---------------------------------------------------------------------------
// Stencil / update.  A block is ST_WARPS warps, one image row each (rows
// y0-1 .. y0+ST_OY; the outer two are halo rows), 32 lanes wide (columns
// x0-1 .. x0+30; lanes 0 and 31 are halo columns), streaming ST_ZC planes.
// Each step computes the gradient / normalised gradient of plane s+1 once
// per thread, exchanges x neighbours by warp shuffles and y neighbours
// through triple-buffered shared rows (one barrier per plane), and writes the
// updated phi of plane s.
// ---------------------------------------------------------------------------
struct GN {
    float gx, gy, gz, nx, ny, nz;
};

template <Arith A>
__device__ __forceinline__ GN gn_from(float xl, float xr, float yl, float yr, float zl, float zr) {
    GN g;
    g.gx = half_diff(xr, xl);
    g.gy = half_diff(yr, yl);
    g.gz = half_diff(zr, zl);
    const NormDen d = norm_den<A>(grad_mag(g.gx, g.gy, g.gz));
    g.nx = normalise<A>(g.gx, d);
    g.ny = normalise<A>(g.gy, d);
    g.nz = normalise<A>(g.gz, d);
    return g;
}

// Gradient and normalised gradient at (x, y, z) straight from global memory
// with the boundary rules of kernel.cu:57-125; used for the previous-row
// neighbour that x = 0 reads in the reference boundary mode.
template <Arith A>
__device__ __noinline__ GN gn_global(const float *__restrict__ phi, int x, int y, int z, int W, int H, int L,
                                     int boundary) {
    const size_t WH = (size_t)W * H;
    auto at = [&](int xx, int yy, int zz) { return __ldg(phi + (size_t)zz * WH + (size_t)yy * W + xx); };
    const float c0 = at(x, y, z);
    float xl;
    if (x > 0) xl = at(x - 1, y, z);
    else if (boundary == 0) {
        if (y > 0) xl = at(W - 1, y - 1, z);
        else if (z > 0) xl = at(W - 1, H - 1, z - 1);
        else xl = c0;
    } else xl = c0;
    const float xr = x < W - 1 ? at(x + 1, y, z) : c0;
    const float yl = y > 0 ? at(x, y - 1, z) : c0, yr = y < H - 1 ? at(x, y + 1, z) : c0;
    const float zl = z > 0 ? at(x, y, z - 1) : c0, zr = z < L - 1 ? at(x, y, z + 1) : c0;
    return gn_from<A>(xl, xr, yl, yr, zl, zr);
}

template <Arith A, bool DEBUG>
__global__ void __launch_bounds__(ST_WARPS * 32, 2) stencil_kernel(const SubVolDev *__restrict__ svs,
                                                                   const int *__restrict__ pre,
                                                                   const StepConst c, int parity,
                                                                   unsigned *__restrict__ flag, DebugOut dbg) {
    __shared__ float Pb[3][ST_WARPS][32];
    __shared__ float Gb[3][2][ST_WARPS][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int W = s.W, H = s.H, L = s.L;
    const int ntx = (W + ST_OX - 1) / ST_OX, nty = (H + ST_OY - 1) / ST_OY;
    const int tx = t % ntx;
    t /= ntx;
    const int ty = t % nty;
    const int tz = t / nty;
    const int x = tx * ST_OX - 1 + lane, y = ty * ST_OY - 1 + w;
    const int z0 = tz * ST_ZC, z1 = min(z0 + ST_ZC, L);
    const bool in = x >= 0 && x < W && y >= 0 && y < H;
    const bool outp = in && lane >= 1 && lane <= ST_OX && w >= 1 && w <= ST_OY;
    const float *__restrict__ phi = parity ? s.phi[1] : s.phi[0];
    float *__restrict__ phi_out = parity ? s.phi[0] : s.phi[1];
    const size_t WH = (size_t)W * H;
    const size_t col = in ? (size_t)y * W + x : 0;
    const bool ref = c.boundary == 0;
    const int r = c.r;
    const bool valid_blur = s.Wv > 0;

    // Neighbour values the shuffles and shared rows cannot supply:
    //   x: lane 0 reads x-1; the column x == 0 reads the previous linear
    //      element in the reference mode; lane 31 reads x+1.
    //   y: warp 0 reads y-1, the last warp reads y+1.
    const bool need_xl = in && (lane == 0 || (x == 0 && ref));
    const bool need_xr = in && lane == 31 && x + 1 < W;
    const bool need_yl = in && w == 0 && y > 0;
    const bool need_yr = in && w == ST_WARPS - 1 && y + 1 < H;
    auto ld = [&](int p) -> float { return (in && p >= 0 && p < L) ? __ldg(phi + (size_t)p * WH + col) : 0.0f; };
    auto ld_xl = [&](int p) -> float {
        if (!need_xl || p < 0 || p >= L) return 0.0f;
        if (x > 0) return __ldg(phi + (size_t)p * WH + col - 1);
        if (y > 0) return __ldg(phi + (size_t)p * WH + (size_t)(y - 1) * W + (W - 1));
        if (p > 0) return __ldg(phi + (size_t)(p - 1) * WH + (size_t)(H - 1) * W + (W - 1));
        return __ldg(phi);
    };
    auto ld_xr = [&](int p) -> float {
        return (need_xr && p >= 0 && p < L) ? __ldg(phi + (size_t)p * WH + col + 1) : 0.0f;
    };
    auto ld_y = [&](int p) -> float {
        if (p < 0 || p >= L) return 0.0f;
        if (need_yl) return __ldg(phi + (size_t)p * WH + col - W);
        if (need_yr) return __ldg(phi + (size_t)p * WH + col + W);
        return 0.0f;
    };
    // data factor of (x, y, p): from the z-pass inside the valid region,
    // f_out = f_in = 30/30 = 1 in the border band.
    auto ld_data = [&](int p) -> float {
        if (!outp || p < 0 || p >= L) return 0.0f;
        const bool inside = valid_blur && x >= r && x < W - r && y >= r && y < H - r && p >= r && p < L - r;
        if (inside) return __ldg(s.db + ((size_t)(p - r) * s.Hv + (y - r)) * s.Wp + (x - r));
        const float I = load_img(s.img, (size_t)p * WH + col, c.img_f32);
        const float d = __fsub_rn(I, 1.0f);
        const float e = __fmul_rn(d, d);
        return data_factor(e, e, c.l1, c.l2, c.lam_equal != 0);
    };
    auto slot = [](int p) { return (p + 3) % 3; };

    // prologue: planes z0-2, z0-1, z0 in registers, row z0-1 shared
    const int sp = z0 - 2;
    float p0 = ld(sp), p1 = ld(sp + 1), p2 = ld(sp + 2);
    float exl = ld_xl(sp + 1), exr = ld_xr(sp + 1), exy = ld_y(sp + 1);
    float exl_n = ld_xl(sp + 2), exr_n = ld_xr(sp + 2), exy_n = ld_y(sp + 2);
    Pb[slot(sp + 1)][w][lane] = p1;
    GN gprev = {0, 0, 0, 0, 0, 0}, gcur = gprev, gnext = gprev;
    float dcur = 0.0f;
    __syncthreads();

    for (int sc = z0 - 2; sc < z1; ++sc) {
        const int pn = sc + 1;  // plane whose gradient this step computes
        // prefetch for the next step
        const float p3 = ld(sc + 3);
        const float exl_nn = ld_xl(sc + 3), exr_nn = ld_xr(sc + 3), exy_nn = ld_y(sc + 3);
        const float dnext = (sc + 1 >= z0 && sc + 1 < z1) ? ld_data(sc + 1) : 0.0f;
        Pb[slot(sc + 2)][w][lane] = p2;
        // neighbours of plane pn
        float L1 = __shfl_up_sync(0xffffffffu, p1, 1);
        float R1 = __shfl_down_sync(0xffffffffu, p1, 1);
        if (need_xl) L1 = exl;
        if (lane == 31) R1 = exr;
        const float U1 = w > 0 ? Pb[slot(pn)][w - 1][lane] : exy;
        const float D1 = w < ST_WARPS - 1 ? Pb[slot(pn)][w + 1][lane] : exy;
        if (in && pn >= 0 && pn < L) {
            const float xl = (x > 0 || ref) ? L1 : p1;
            const float xr = x < W - 1 ? R1 : p1;
            const float yl = y > 0 ? U1 : p1, yr = y < H - 1 ? D1 : p1;
            const float zl = pn > 0 ? p0 : p1, zr = pn < L - 1 ? p2 : p1;
            gnext = gn_from<A>(xl, xr, yl, yr, zl, zr);
        } else {
            gnext = GN{0, 0, 0, 0, 0, 0};
        }
        Gb[slot(pn)][0][w][lane] = gnext.ny;
        Gb[slot(pn)][1][w][lane] = gnext.gy;
        __syncthreads();
        // output plane sc
        const float nxL = __shfl_up_sync(0xffffffffu, gcur.nx, 1), nxR = __shfl_down_sync(0xffffffffu, gcur.nx, 1);
        const float gxL = __shfl_up_sync(0xffffffffu, gcur.gx, 1), gxR = __shfl_down_sync(0xffffffffu, gcur.gx, 1);
        if (sc >= z0 && outp) {
            float nxl = nxL, gxl = gxL;
            if (x == 0) {
                if (ref && (y > 0 || sc > 0)) {
                    const GN wg = y > 0 ? gn_global<A>(phi, W - 1, y - 1, sc, W, H, L, c.boundary)
                                        : gn_global<A>(phi, W - 1, H - 1, sc - 1, W, H, L, c.boundary);
                    nxl = wg.nx;
                    gxl = wg.gx;
                } else {
                    nxl = gcur.nx;
                    gxl = gcur.gx;
                }
            }
            const float nxr = x < W - 1 ? nxR : gcur.nx, gxr = x < W - 1 ? gxR : gcur.gx;
            const int so = slot(sc);
            const float nyl = y > 0 ? Gb[so][0][w - 1][lane] : gcur.ny;
            const float nyr = y < H - 1 ? Gb[so][0][w + 1][lane] : gcur.ny;
            const float gyl = y > 0 ? Gb[so][1][w - 1][lane] : gcur.gy;
            const float gyr = y < H - 1 ? Gb[so][1][w + 1][lane] : gcur.gy;
            const float nzl = sc > 0 ? gprev.nz : gcur.nz, nzr = sc < L - 1 ? gnext.nz : gcur.nz;
            const float gzl = sc > 0 ? gprev.gz : gcur.gz, gzr = sc < L - 1 ? gnext.gz : gcur.gz;
            const float kap = __fadd_rn(__fadd_rn(half_diff(nxr, nxl), half_diff(nyr, nyl)), half_diff(nzr, nzl));
            const float lap = __fadd_rn(__fadd_rn(half_diff(gxr, gxl), half_diff(gyr, gyl)), half_diff(gzr, gzl));
            const float dh = dirac<A>(p0, c.eps);
            const float out = update_phi(p0, dh, dcur, kap, lap, c.dt, c.nu, c.mu);
            const size_t vi = (size_t)sc * WH + col;
            phi_out[vi] = out;
            if (!isfinite(out)) atomicOr(flag, 1u);
            if constexpr (DEBUG) {
                const bool inside = valid_blur && x >= r && x < W - r && y >= r && y < H - r && sc >= r && sc < L - r;
                if (!inside) {
                    const float I = load_img(s.img, vi, c.img_f32);
                    const float d = __fsub_rn(I, 1.0f);
                    dbg.f[0 * dbg.n + vi] = 1.0f;
                    dbg.f[1 * dbg.n + vi] = 1.0f;
                    dbg.f[2 * dbg.n + vi] = __fmul_rn(d, d);
                    dbg.f[3 * dbg.n + vi] = __fmul_rn(d, d);
                }
                dbg.f[4 * dbg.n + vi] = dh;
                dbg.f[5 * dbg.n + vi] = kap;
                dbg.f[6 * dbg.n + vi] = lap;
                dbg.f[7 * dbg.n + vi] = grad_mag(gcur.gx, gcur.gy, gcur.gz);
            }
        }
        p0 = p1;
        p1 = p2;
        p2 = p3;
        exl = exl_n;
        exr = exr_n;
        exy = exy_n;
        exl_n = exl_nn;
        exr_n = exr_nn;
        exy_n = exy_nn;
        gprev = gcur;
        gcur = gnext;
        dcur = dnext;
    }
}

}  // namespace rsf
