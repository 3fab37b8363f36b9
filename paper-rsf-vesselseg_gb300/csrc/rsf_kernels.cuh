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
    const int ntx = (s.Wv + XT - 1) / XT, nty = (s.H + XP_ROWS * c.xrpw - 1) / (XP_ROWS * c.xrpw);
    const int tx = t % ntx;
    t /= ntx;
    const int ty = t % nty;
    const int z = t / nty;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float2 *taps_s = reinterpret_cast<float2 *>(sm4 + XP_ROWS * span);  // MAXK pairs, then the pair-0 stages
    if (K == 0) {
        for (int i = threadIdx.x; i < k; i += blockDim.x) taps_s[i] = c.taps2[i];
        __syncthreads();
    }
    float4 *in = sm4 + warp * span;
    const int x0 = tx * XT;
    // c.xrpw rows per warp, XP_ROWS apart: the block setup above is paid
    // once per c.xrpw row segments
    for (int j = 0; j < c.xrpw; ++j) {
        const int y = (ty * c.xrpw + j) * XP_ROWS + warp;
        if (y >= s.H) break;
        if (j > 0) __syncwarp();  // the previous row's stores have read the slab
        const size_t row = ((size_t)z * s.H + y) * s.W;
        const float *phi = (parity ? s.phi[1] : s.phi[0]) + row;
        if constexpr (K > 0) {
            // all of the lane's loads first, so that they are in flight together
            constexpr int NE = (XT + K - 1 + 31) / 32;
            float ph[NE], im[NE];
#pragma unroll
            for (int q = 0; q < NE; ++q) {
                const int e = lane + 32 * q, x = x0 + e;
                const bool ok = e < span && x < s.W;
                ph[q] = ok ? __ldg(phi + x) : 0.0f;
                im[q] = ok ? load_img(s.img, row + x, c.img_f32) : 0.0f;
            }
#pragma unroll
            for (int q = 0; q < NE; ++q) {
                const int e = lane + 32 * q;
                if (e < span) {
                    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (x0 + e < s.W) {
                        const float h = heaviside<A>(ph[q], c.eps);
                        const float hi = __fsub_rn(1.0f, h);
                        v = make_float4(h, hi, __fmul_rn(im[q], h), __fmul_rn(im[q], hi));
                    }
                    in[e] = v;
                }
            }
        } else {
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
        }
        __syncwarp();
        // Pair 0 (H, 1-H) is staged in its own slab, pair 1 (I H, I (1-H)) in
        // the input slab once every lane has finished reading it.
        float *st01 = reinterpret_cast<float *>(sm4 + XP_ROWS * span) + 2 * MAXK + warp * 2 * XT;
        float *st23 = reinterpret_cast<float *>(in);
        const float2 *src = reinterpret_cast<const float2 *>(in + XB * lane);
        float2 acc[XB];
        if constexpr (K > 0) {
            // two float2 pair planes: each pair's results are staged as float2
            // and written as float4 (two columns)
            float2 *s01 = reinterpret_cast<float2 *>(st01), *s23 = reinterpret_cast<float2 *>(st23);
            xconv_pair<K, XB>(src, c, taps_s, k, acc);
#pragma unroll
            for (int m = 0; m < XB; ++m) s01[XB * lane + m] = acc[m];
            xconv_pair<K, XB>(src + 1, c, taps_s, k, acc);
            __syncwarp();
#pragma unroll
            for (int m = 0; m < XB; ++m) s23[XB * lane + m] = acc[m];
            __syncwarp();
            const size_t pstride = (size_t)s.Wp * s.H * s.L;
            const size_t orow = ((size_t)z * s.H + y) * s.Wp;
#pragma unroll
            for (int pp = 0; pp < 2; ++pp) {
                const float4 *sf = reinterpret_cast<const float4 *>(pp ? s23 : s01);
                float4 *dst = reinterpret_cast<float4 *>(reinterpret_cast<float2 *>(s.xb) + pp * pstride + orow + x0);
                for (int e = lane; e < XT / 2; e += 32)
                    if (x0 + 2 * e < s.Wv) dst[e] = sf[e];
            }
        } else {
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
    }
}

// ---------------------------------------------------------------------------
// Streaming valid correlation along a strided axis for a pair of columns:
// inputs src[i * stride] for i in [0, n), outputs o = i - K + 1 in [0, n-K+1)
// handed to emit(o, value) as soon as they complete.
// ---------------------------------------------------------------------------
// Inputs reach the thread through a private ring of RING float2 slots in
// shared memory filled by cp.async, so that RING loads per thread are in
// flight while the multiply-adds run.  Element i lives in slot i % RING and
// in commit group i; iteration i first refills the slot element i-1 used
// (with element i-1+RING, group RING+i-1), then waits until at most RING-1
// groups are pending, which completes group i.
constexpr int RING = 8;

__device__ __forceinline__ void cp_async8(float2 *smem_dst, const float *gsrc) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async4(unsigned *smem_dst, const void *gsrc) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_ring() { asm volatile("cp.async.wait_group %0;" ::"n"(RING - 1) : "memory"); }

struct Ring {
    float2 *base;     // this thread's slot 0; slot s at base + s * step
    int step;         // threads per block
    const float *src; // element i at src + i * stride
    size_t stride;
    int n;
    bool act;         // inactive threads load nothing (their results are discarded)
    // Optional side stream riding in the same commit groups: with element i
    // comes the aligned 32-bit word holding byte side + (i - lag) * sstride,
    // for i >= first.  The word around a valid byte stays inside that byte's
    // 4-byte-aligned block, so it never touches another allocation.
    unsigned *sbase = nullptr;
    const unsigned char *side = nullptr;
    size_t sstride = 0;
    int lag = 0, first = 0;
    bool sact = false;
    __device__ __forceinline__ float2 *slot(int i) const { return base + (i & (RING - 1)) * step; }
    __device__ __forceinline__ unsigned *sslot(int i) const { return sbase + (i & (RING - 1)) * step; }
    __device__ __forceinline__ const unsigned char *sbyte(int i) const { return side + (size_t)(i - lag) * sstride; }
    __device__ __forceinline__ void fill(int i) const {
        if (act && i < n) {
            cp_async8(slot(i), src + (size_t)i * stride);
            if (sact && i >= first)
                cp_async4(sslot(i),
                          reinterpret_cast<const void *>(reinterpret_cast<uintptr_t>(sbyte(i)) & ~(uintptr_t)3));
        }
    }
};

template <int K, bool GUARD, typename Emit>
__device__ __forceinline__ void stream_block(const Ring &rg, int base, const StepConst &c, float2 (&acc)[K],
                                             Emit &emit) {
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const int i = base + j;
        if (GUARD && i >= rg.n) break;
        if (i > 0) {
            rg.fill(i - 1 + RING);
            cp_commit();
        }
        cp_wait_ring();
        const float2 v = *rg.slot(i);
#pragma unroll
        for (int tt = 0; tt < K; ++tt) {
            const int slot = (j - tt + K) % K;
            if (tt == 0) acc[slot] = fma2(v, c.taps2[0], make_float2(0.f, 0.f));
            else acc[slot] = fma2(v, c.taps2[tt], acc[slot]);
        }
        const int o = i - (K - 1);
        if (o >= 0) emit(o, acc[(j + 1) % K], i);
    }
}

template <int K, typename Emit>
__device__ __forceinline__ void stream_axis(const Ring &rg, const StepConst &c, Emit &emit) {
#pragma unroll
    for (int q = 0; q < RING; ++q) {
        rg.fill(q);
        cp_commit();
    }
    float2 acc[K];
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] = make_float2(0.f, 0.f);
    int base = 0;
    for (; base + K <= rg.n; base += K) stream_block<K, false>(rg, base, c, acc, emit);
    if (base < rg.n) stream_block<K, true>(rg, base, c, acc, emit);
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// Ring with compile-time slots, for tap counts that are a multiple of the
// ring depth RD (21 and 35 with RD = 7, 29 with RD = 29).  Blocks of K
// elements start at multiples of K, so element base + j sits in slot j % RD,
// a constant of the unrolled block; the global addresses advance by one stride per element
// instead of being recomputed.  Same commit-group protocol as Ring: element
// i is group i; iteration i refills the slot of element i-1 with element
// i-1+RD and then waits until at most RD-1 groups are pending.
template <int RD>
__device__ __forceinline__ void cp_wait_depth() {
    asm volatile("cp.async.wait_group %0;" ::"n"(RD - 1) : "memory");
}

template <int RD>
struct RingC {
    float2 *base;              // this thread's slot 0; slot q at base + q * step
    int step;
    const float *next;         // global address of element `nfill`
    size_t stride;
    int nfill, n;
    bool act;
    // side stream: the aligned word around byte snext for elements >= sfirst
    unsigned *sbase = nullptr;
    const unsigned char *snext = nullptr;
    size_t sstride = 0;
    int sfirst = 0;
    bool sact = false;
    // `slot` is a constant after the caller's loop is unrolled
    __device__ __forceinline__ void fill(int slot) {
        if (act && nfill < n) {
            cp_async8(base + slot * step, next);
            if (sact && nfill >= sfirst)
                cp_async4(sbase + slot * step,
                          reinterpret_cast<const void *>(reinterpret_cast<uintptr_t>(snext) & ~(uintptr_t)3));
        }
        next += stride;  // addresses past the end are formed but never read
        if (nfill >= sfirst) snext += sstride;
        ++nfill;
    }
};

template <int K, int RD, bool FIRST, bool GUARD, typename Emit>
__device__ __forceinline__ void stream_block_c(RingC<RD> &rg, int base, const StepConst &c, float2 (&acc)[K],
                                               Emit &emit) {
    static_assert(K % RD == 0, "the ring depth must divide the tap count");
#pragma unroll
    for (int j = 0; j < K; ++j) {
        if (GUARD && base + j >= rg.n) break;
        if (!(FIRST && j == 0)) {
            rg.fill((j - 1 + RD) % RD);
            cp_commit();
        }
        cp_wait_depth<RD>();
        const float2 v = rg.base[(j % RD) * rg.step];
#pragma unroll
        for (int tt = 0; tt < K; ++tt) {
            const int slot = (j - tt + K) % K;
            if (tt == 0) acc[slot] = fma2(v, c.taps2[0], make_float2(0.f, 0.f));
            else acc[slot] = fma2(v, c.taps2[tt], acc[slot]);
        }
        if (!FIRST || j >= K - 1) emit(base + j - (K - 1), acc[(j + 1) % K], j % RD);
    }
}

template <int K, int RD, typename Emit>
__device__ __forceinline__ void stream_axis_c(RingC<RD> &rg, const StepConst &c, Emit &emit) {
#pragma unroll
    for (int q = 0; q < RD; ++q) {
        rg.fill(q);
        cp_commit();
    }
    float2 acc[K];
#pragma unroll
    for (int j = 0; j < K; ++j) acc[j] = make_float2(0.f, 0.f);
    if (rg.n < K) {
        stream_block_c<K, RD, true, true>(rg, 0, c, acc, emit);
    } else {
        stream_block_c<K, RD, true, false>(rg, 0, c, acc, emit);
        int base = K;
        for (; base + K <= rg.n; base += K) stream_block_c<K, RD, false, false>(rg, base, c, acc, emit);
        if (base < rg.n) stream_block_c<K, RD, false, true>(rg, base, c, acc, emit);
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// Depth of the compile-time ring of a specialised tap count: 7 for 21 and
// 35; 29 (prime) takes a ring as deep as its taps (44.5 KB of shared memory
// per block, within what its registers already allow per SM).
__host__ __device__ constexpr int ring_depth(int K) { return K % 7 == 0 ? 7 : K == 29 ? 29 : RING; }

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
// y-pass.  One thread streams one column of one pair plane of one z plane
// (float2 elements: both fields of the pair, one packed multiply-add).
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(YP_COLS) ypass_kernel(const SubVolDev *__restrict__ svs,
                                                        const int *__restrict__ pre, const StepConst c) {
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int ntx = (s.Wv + YP_COLS - 1) / YP_COLS;
    const int tx = t % ntx;
    t /= ntx;
    const int p = t & 1;
    const int z = t >> 1;
    __shared__ float2 ring[RING * YP_COLS];
    const int x = tx * YP_COLS + threadIdx.x;
    if (x >= s.Wv) return;
    const float *src = s.xb + 2 * ((size_t)p * s.Wp * s.H * s.L + (size_t)z * s.H * s.Wp + x);
    float2 *dst = reinterpret_cast<float2 *>(s.yb) + (size_t)p * s.Wp * s.Hv * s.L + (size_t)z * s.Hv * s.Wp + x;
    const size_t wp = (size_t)s.Wp;
    // The y-pass is bound by HBM bandwidth: it keeps the deeper 8-slot ring
    // (more loads in flight) rather than the compile-time-slot ring.
    auto emit = [&](int o, float2 v, int) { dst[(size_t)o * wp] = v; };
    const Ring rg = {ring + threadIdx.x, YP_COLS, src, 2 * wp, s.H, true};
    stream_axis<K>(rg, c, emit);
}

// U = 1: the second (expanded data term) pass, reading the scratch G at
// xb + gdelta instead of the x-pass fields.
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
    const float *src = (U ? s.xb + c.gdelta : s.xb) + f * ((size_t)s.Wp * s.H * s.L) + (size_t)z * s.H * s.Wp + x;
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
// x column of lane f of a 4-lane group (column pair x, x+1): with the four
// separate y fields lane f streams field f of both columns; with the pair
// layout lane f streams pair f >> 1 of column x + (f & 1).
template <bool PAIRS>
__device__ __forceinline__ int zlane_col(int x, int f) {
    return PAIRS ? x + (f & 1) : x + (f >> 1);
}

template <bool PAIRS>
__device__ __forceinline__ void fits_and_data(const SubVolDev &s, const StepConst &c, int f, int x, int y, int o,
                                              bool live, float I, float2 B, const DebugOut &dbg, bool debug) {
    // Separate fields: B = (field f at x, field f at x+1); lane f forms
    //   0 -> f_out(x), 1 -> f_in(x), 2 -> f_out(x+1), 3 -> f_in(x+1).
    // Pair layout: B = (pair f>>1 at column x + (f&1)); lane f forms
    //   0 -> f_out(x), 1 -> f_out(x+1), 2 -> f_in(x), 3 -> f_in(x+1).
    // Both are num / den with num = lane f+2's B.x for f < 2, else B.y, and
    // den = B.x for f < 2, else lane f-2's B.y.  I is the image at the
    // lane's voxel (prefetched by the caller).
    const float bx_hi = __shfl_down_sync(0xffffffffu, B.x, 2);
    const float by_lo = __shfl_up_sync(0xffffffffu, B.y, 2);
    const float num = f < 2 ? bx_hi : B.y;
    const float den = f < 2 ? B.x : by_lo;
    const float fv = __fdiv_rn(num, den);
    const int xc = zlane_col<PAIRS>(x, f);
    const float d = __fsub_rn(I, fv);
    const float e = __fmul_rn(d, d);
    // the lane holding f_out of a column gets that column's e_in
    const float e_in = __shfl_down_sync(0xffffffffu, e, PAIRS ? 2 : 1);
    const bool outer = PAIRS ? f < 2 : (f & 1) == 0;
    if (live && outer)
        s.db[((size_t)o * s.Hv + y) * s.Wp + xc] = data_factor(e, e_in, c.l1, c.l2, c.lam_equal != 0);
    if (debug && live) {
        const int r = c.r;
        const int fin = outer ? 0 : 1;
        const size_t vi = ((size_t)(o + r) * s.H + (y + r)) * s.W + (xc + r);
        dbg.f[(size_t)fin * dbg.n + vi] = fv;
        dbg.f[(size_t)(2 + fin) * dbg.n + vi] = e;
    }
}

// The streaming z-pass of one block (tile t of sub-volume s): every lane
// gets its column's blurred pair at each output plane o and the image there,
// and hands them to fits(f, x, y, o, live, I, B), which all lanes of the warp
// call together (it may shuffle), for o = 0, 1, ..., Lv - 1 in order.
// begin(xc, y, live) runs first, with the lane's output column xc.
template <int K, bool PAIRS, class Begin, class Fits>
__device__ __forceinline__ void zpass_body(const SubVolDev &s, const StepConst &c, int t, Begin begin, Fits fits) {
    const int ntx = (s.Wv + 2 * ZP_PAIRS - 1) / (2 * ZP_PAIRS);
    const int tx = t % ntx;
    const int y = t / ntx;
    const int f = threadIdx.x & 3;
    const int x = 2 * (tx * ZP_PAIRS + (threadIdx.x >> 2));
    const bool act = x < s.Wv;
    // separate fields: field f, column pair x; pair layout: pair f >> 1,
    // column x + (f & 1), float2 elements (plane stride in floats doubles)
    const float *src = PAIRS ? s.yb + (size_t)(f >> 1) * 2 * ((size_t)s.Wp * s.Hv * s.L) +
                                   2 * ((size_t)y * s.Wp + (act ? x + (f & 1) : 0))
                             : s.yb + f * ((size_t)s.Wp * s.Hv * s.L) + (size_t)y * s.Wp + (act ? x : 0);
    const size_t pstride = (PAIRS ? 2 : 1) * (size_t)s.Wp * s.Hv;
    constexpr int RS = ring_depth(K) > RING ? ring_depth(K) : RING;
    __shared__ float2 ring[RS * ZP_PAIRS * 4];
    __shared__ unsigned iring[RS * ZP_PAIRS * 4];
    // The image at this lane's voxel of output plane o (input plane o + r)
    // rides in the ring with element i = o + 2r.
    const int xc = zlane_col<PAIRS>(x, f);
    const bool live = act && xc < s.Wv;
    const size_t esz = c.img_f32 ? 4 : 1;
    const unsigned char *img0 = static_cast<const unsigned char *>(s.img) +
                                (((size_t)(y + c.r)) * s.W + (size_t)(xc + c.r)) * esz;
    const size_t sstride = (size_t)s.W * s.H * esz;
    begin(xc, y, live);
    if constexpr (K % ring_depth(K) == 0 && ring_depth(K) != RING) {
        constexpr int RD = ring_depth(K);
        RingC<RD> rg = {ring + threadIdx.x, ZP_PAIRS * 4, src, pstride, 0, s.L, act};
        rg.sbase = iring + threadIdx.x;
        rg.snext = img0 + (size_t)c.r * sstride;  // element 2r carries plane r, the first output's
        rg.sstride = sstride;
        rg.sfirst = 2 * c.r;
        rg.sact = live;
        // low two bits of the byte address of output o's image voxel:
        // (shift0 + o * sstride) mod 4
        const unsigned shift0 = (unsigned)(reinterpret_cast<uintptr_t>(img0 + (size_t)c.r * sstride) & 3);
        const unsigned shift_step = (unsigned)(sstride & 3);
        auto emit = [&](int o, float2 v, int slot) {
            float I = 0.0f;
            if (live) {
                const unsigned wd = rg.sbase[slot * rg.step];
                if (c.img_f32) I = __uint_as_float(wd);
                else I = (float)((wd >> (8 * ((shift0 + (unsigned)o * shift_step) & 3u))) & 0xffu);
            }
            fits(f, x, y, o, live, I, v);
        };
        stream_axis_c<K, RD>(rg, c, emit);
    } else {
        Ring rg = {ring + threadIdx.x, ZP_PAIRS * 4, src, pstride, s.L, act};
        rg.sbase = iring + threadIdx.x;
        rg.side = img0;
        rg.sstride = sstride;
        rg.lag = c.r;
        rg.first = 2 * c.r;
        rg.sact = live;
        auto emit = [&](int o, float2 v, int i) {
            float I = 0.0f;
            if (live) {
                const unsigned wd = *rg.sslot(i);
                if (c.img_f32) I = __uint_as_float(wd);
                else I = (float)((wd >> (8 * (unsigned)(reinterpret_cast<uintptr_t>(rg.sbyte(i)) & 3))) & 0xffu);
            }
            fits(f, x, y, o, live, I, v);
        };
        stream_axis<K>(rg, c, emit);
    }
}

template <int K, bool DEBUG, bool PAIRS = false>
__global__ void __launch_bounds__(ZP_PAIRS * 4) zpass_kernel(const SubVolDev *__restrict__ svs,
                                                             const int *__restrict__ pre, const StepConst c,
                                                             DebugOut dbg) {
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    zpass_body<K, PAIRS>(
        s, c, b - __ldg(pre + sv), [](int, int, bool) {},
        [&](int f, int x, int y, int o, bool live, float I, float2 v) {
            fits_and_data<PAIRS>(s, c, f, x, y, o, live, I, v, dbg, DEBUG);
        });
}

// The same z-pass bounded only to two resident blocks per SM.  For 35 taps
// the default bounds hold it to 128 registers with a 56-byte spill of the 35
// accumulator pairs; this one takes 164 registers without a spill (3 blocks
// per SM instead of 4) and measured 1.43 against 1.89 ms per launch on a
// 512^3 volume.
template <int K, bool PAIRS>
__global__ void __launch_bounds__(ZP_PAIRS * 4, 2) zpass_wide_kernel(const SubVolDev *__restrict__ svs,
                                                                     const int *__restrict__ pre,
                                                                     const StepConst c) {
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    const DebugOut none = {nullptr, 0};
    zpass_body<K, PAIRS>(
        s, c, b - __ldg(pre + sv), [](int, int, bool) {},
        [&](int f, int x, int y, int o, bool live, float I, float2 v) {
            fits_and_data<PAIRS>(s, c, f, x, y, o, live, I, v, none, false);
        });
}

// The adjoint's recompute of the fits (rsf_adjoint.cu): the forward z-pass
// over pair planes, emitting at each valid voxel, instead of the data factor,
//   e_out = (I - f_out)^2 and e_in at the full-volume index, and the pair
//   (B1_bar - B3_bar, B2_bar - B4_bar) in the valid layout (row stride Wv),
// with B1..B4 the blurs of I H, H, I (1-H), 1-H, f_out = B1 / B2,
// f_in = B3 / B4, and for data_bar = -u dt delta(phi)
//   f_out_bar = -2 (I - f_out) lambda1 data_bar, f_in_bar = 2 (I - f_in) lambda2 data_bar,
//   B1_bar = f_out_bar / B2, B2_bar = -f_out_bar f_out / B2 (B3, B4 alike).
// ph, uo: phi and u at the lane's voxel of output plane o.  The pair goes to
// a.xs (2 Wv Hv Lv floats), e_out and e_in to a.xs + 2 N and a.xs + 3 N.
__device__ __forceinline__ void adjoint_fits(const SubVolDev &s, const StepConst &c, const AdjVol &a, int f, int x,
                                             int y, int o, bool live, float I, float2 B, float ph, float uo) {
    // lanes as in fits_and_data's pair layout: 0, 1 -> f_out at x, x + 1;
    // 2, 3 -> f_in at x, x + 1
    const float bx_hi = __shfl_down_sync(0xffffffffu, B.x, 2);
    const float by_lo = __shfl_up_sync(0xffffffffu, B.y, 2);
    const bool outer = f < 2;
    const float num = outer ? bx_hi : B.y;
    const float den = outer ? B.x : by_lo;
    const int xc = x + (f & 1);
    const size_t vi = ((size_t)(o + c.r) * s.H + (y + c.r)) * s.W + (xc + c.r);
    float bn = 0.0f, bd = 0.0f, e = 0.0f;
    if (live) {
        const float rb = __frcp_rn(den);
        const float fv = num * rb;
        const float d = I - fv;
        e = d * d;
        const float delta = __fdividef(0.318309886183790672f * c.eps, fmaf(ph, ph, c.eps * c.eps));
        const float data_bar = -uo * c.dt * delta;
        const float fbar = -2.0f * d * (outer ? c.l1 * data_bar : -c.l2 * data_bar);
        bn = fbar * rb;
        bd = -fbar * fv * rb;
    }
    const float bn_in = __shfl_down_sync(0xffffffffu, bn, 2);
    const float bd_in = __shfl_down_sync(0xffffffffu, bd, 2);
    if (live) {
        const size_t n = (size_t)s.W * s.H * s.L;
        if (outer) {
            const size_t nv = (size_t)s.Wv * s.Hv * s.Lv;
            const size_t vo = ((size_t)o * s.Hv + y) * s.Wv + xc;
            a.xs[vo] = bn - bn_in;
            a.xs[nv + vo] = bd - bd_in;
            a.xs[2 * n + vi] = e;
        } else {
            a.xs[3 * n + vi] = e;
        }
    }
}

template <int K>
__global__ void __launch_bounds__(ZP_PAIRS * 4) zpass_adjoint_kernel(const SubVolDev *__restrict__ svs,
                                                                     const int *__restrict__ pre, const StepConst c,
                                                                     const AdjVol *__restrict__ vols) {
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    const AdjVol a = vols[sv];
    // phi and u of output planes o, o + 1, o + 2 ride in registers: each
    // output's loads are issued three planes ahead (the streaming loop is
    // latency-bound when the volume gives few blocks per SM).
    const size_t plane = (size_t)s.W * s.H;
    float p0 = 0.f, p1 = 0.f, p2 = 0.f, u0 = 0.f, u1 = 0.f, u2 = 0.f;
    size_t vnext = 0;  // offset of the lane's voxel in plane o + 3 + r
    auto begin = [&](int xc, int y, bool live) {
        const size_t v0 = ((size_t)c.r * s.H + (y + c.r)) * s.W + (xc + c.r);
        if (live) {
            p0 = __ldg(a.phi + v0);
            u0 = __ldg(a.u + v0);
            if (s.Lv > 1) {
                p1 = __ldg(a.phi + v0 + plane);
                u1 = __ldg(a.u + v0 + plane);
            }
            if (s.Lv > 2) {
                p2 = __ldg(a.phi + v0 + 2 * plane);
                u2 = __ldg(a.u + v0 + 2 * plane);
            }
        }
        vnext = v0 + 3 * plane;
    };
    zpass_body<K, true>(s, c, b - __ldg(pre + sv), begin,
                        [&](int f, int x, int y, int o, bool live, float I, float2 v) {
                            const float ph = p0, uo = u0;
                            p0 = p1;
                            u0 = u1;
                            p1 = p2;
                            u1 = u2;
                            if (live && o + 3 < s.Lv) {
                                p2 = __ldg(a.phi + vnext);
                                u2 = __ldg(a.u + vnext);
                            }
                            vnext += plane;
                            adjoint_fits(s, c, a, f, x, y, o, live, I, v, ph, uo);
                        });
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
        if (c.full_data) {  // the box or expanded data-term kernels form e from the fits
            const size_t di = ((size_t)o * s.Hv + y) * s.Wp + x;
            s.db[di] = fo[m];
            s.db[(size_t)s.Wp * s.Hv * s.Lv + di] = fi[m];
            if (DEBUG) {
                dbg.f[0 * dbg.n + vi] = fo[m];
                dbg.f[1 * dbg.n + vi] = fi[m];
            }
            continue;
        }
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
// x0-1 .. x0+30; lanes 0 and 31 are halo columns), streaming c.zc planes.
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
__device__ __forceinline__ GN gn_global(const float *__restrict__ phi, int x, int y, int z, int W, int H, int L,
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

// Per-block state of the stencil kernel.  Planes are numbered relative to
// the block's first step; every ring below is indexed by (relative plane mod
// 3), which the 3-way unrolled step loop turns into compile-time register and
// shared-memory slots.
struct StencilCtx {
    const SubVolDev *s;
    const float *phi;       // this thread's column of phi (plane 0 at offset 0)
    float *phi_out;
    const float *dcol;      // this thread's column of the data factor (plane r)
    size_t WH, dplane;
    int W, H, L, r, x, y, w, lane, z0, z1, first;
    bool in, outp, ref, inside_xy, blk_inside;
    bool need_x, need_y;
    ptrdiff_t xoff, yoff;   // offsets of the extra neighbour loads
    size_t col;
    // fast path (stencil_step_f): rows of the y neighbours in the shared
    // rings, and the x face rules of the thread's voxel
    int urow, drow;         // phi rows above / below (Pb, ST_WARPS + 2 rows)
    int gwl, gwr;           // gradient rows above / below (Gb)
    bool xl_self, xr_self;  // the x - 1 / x + 1 neighbour is the voxel itself
};

// nx, gx, nz, gz of a plane (ny, gy live in the shared rows)
struct GN4 {
    float nx, gx, nz, gz;
};

struct StencilState {
    float P[3];     // phi of the planes
    float EX[3];    // extra x neighbour
    float EY[3];    // extra y neighbour
    float DT[3];    // data factor of the planes
    GN4 G[3];       // gradient / normalised gradient of the planes
};

__device__ __forceinline__ float st_ld(const StencilCtx &k, int p) {
    return (k.in && p >= 0 && p < k.L) ? __ldg(k.phi + (size_t)p * k.WH) : 0.0f;
}
__device__ __forceinline__ float st_ldx(const StencilCtx &k, int p) {
    if (!k.need_x || p < 0 || p >= k.L) return 0.0f;
    // previous linear element of voxel 0 is defined as voxel 0 itself
    if (k.xoff < 0 && p == 0 && k.col == 0) return __ldg(k.phi);
    return __ldg(k.phi + (ptrdiff_t)((size_t)p * k.WH) + k.xoff);
}
__device__ __forceinline__ float st_ldy(const StencilCtx &k, int p) {
    return (k.need_y && p >= 0 && p < k.L) ? __ldg(k.phi + (ptrdiff_t)((size_t)p * k.WH) + k.yoff) : 0.0f;
}
// data factor at plane p: from the z-pass inside the valid region, from
// f_out = f_in = 30/30 = 1 in the border band (kernel.cu:300-325).
__device__ __forceinline__ float st_data(const StencilCtx &k, const StepConst &c, int p) {
    if (!k.outp || p < k.z0 || p >= k.z1) return 0.0f;
    if (k.blk_inside || (k.inside_xy && p >= k.r && p < k.L - k.r))
        return __ldg(k.dcol + (ptrdiff_t)((size_t)p * k.dplane) - (ptrdiff_t)((size_t)k.r * k.dplane));
    const float I = load_img(k.s->img, (size_t)p * k.WH + k.col, c.img_f32);
    const float d = __fsub_rn(I, 1.0f);
    const float e = __fmul_rn(d, d);
    return data_factor(e, e, c.l1, c.l2, c.lam_equal != 0);
}

template <int C, Arith A, bool DEBUG>
__device__ __forceinline__ void stencil_step(const StencilCtx &k, const StepConst &c, StencilState &S, int rel,
                                             float (*Pb)[ST_WARPS + 2][32], float2 (*Gb)[ST_WARPS][32],
                                             unsigned *flag, const DebugOut &dbg) {
    constexpr int C1 = (C + 1) % 3, C2 = (C + 2) % 3;
    const int sc = k.first + rel;  // output plane of this step
    const int pn = sc + 1;         // plane whose gradient this step computes
    // prefetch for the next steps
    const float p3 = st_ld(k, sc + 3);
    const float exn = st_ldx(k, sc + 3), eyn = st_ldy(k, sc + 3);
    const float dn = st_data(k, c, sc + 1);
    Pb[C2][k.w + 1][k.lane] = S.P[C2];
    const float p0 = S.P[C], p1 = S.P[C1], p2 = S.P[C2];
    float L1 = __shfl_up_sync(0xffffffffu, p1, 1);
    float R1 = __shfl_down_sync(0xffffffffu, p1, 1);
    if (k.need_x && k.xoff < 0) L1 = S.EX[C1];
    if (k.need_x && k.xoff > 0) R1 = S.EX[C1];
    const float U1 = k.w > 0 ? Pb[C1][k.w][k.lane] : S.EY[C1];
    const float D1 = k.w < ST_WARPS - 1 ? Pb[C1][k.w + 2][k.lane] : S.EY[C1];
    GN gn = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (k.in && pn >= 0 && pn < k.L) {
        const float xl = (k.x > 0 || k.ref) ? L1 : p1;
        const float xr = k.x < k.W - 1 ? R1 : p1;
        const float yl = k.y > 0 ? U1 : p1, yr = k.y < k.H - 1 ? D1 : p1;
        const float zl = pn > 0 ? p0 : p1, zr = pn < k.L - 1 ? p2 : p1;
        gn = gn_from<A>(xl, xr, yl, yr, zl, zr);
    }
    S.G[C1] = GN4{gn.nx, gn.gx, gn.nz, gn.gz};
    Gb[C1][k.w][k.lane] = make_float2(gn.ny, gn.gy);
    __syncthreads();
    const GN4 &gc = S.G[C];
    const float nxL = __shfl_up_sync(0xffffffffu, gc.nx, 1), nxR = __shfl_down_sync(0xffffffffu, gc.nx, 1);
    const float gxL = __shfl_up_sync(0xffffffffu, gc.gx, 1), gxR = __shfl_down_sync(0xffffffffu, gc.gx, 1);
    if (sc >= k.z0 && k.outp) {
        float nxl = nxL, gxl = gxL;
        if (k.x == 0) {
            if (k.ref && (k.y > 0 || sc > 0)) {
                const float *phi0 = k.phi - k.col;  // plane 0, voxel 0
                const GN wg = k.y > 0 ? gn_global<A>(phi0, k.W - 1, k.y - 1, sc, k.W, k.H, k.L, c.boundary)
                                      : gn_global<A>(phi0, k.W - 1, k.H - 1, sc - 1, k.W, k.H, k.L, c.boundary);
                nxl = wg.nx;
                gxl = wg.gx;
            } else {
                nxl = gc.nx;
                gxl = gc.gx;
            }
        }
        const bool xr_in = k.x < k.W - 1;
        const float nxr = xr_in ? nxR : gc.nx, gxr = xr_in ? gxR : gc.gx;
        const int wl = k.y > 0 ? k.w - 1 : k.w, wr = k.y < k.H - 1 ? k.w + 1 : k.w;
        const float2 yl2 = Gb[C][wl][k.lane], yr2 = Gb[C][wr][k.lane];
        const float nyl = yl2.x, nyr = yr2.x, gyl = yl2.y, gyr = yr2.y;
        const GN4 &gp = S.G[C2];
        const float nzl = sc > 0 ? gp.nz : gc.nz, nzr = sc < k.L - 1 ? gn.nz : gc.nz;
        const float gzl = sc > 0 ? gp.gz : gc.gz, gzr = sc < k.L - 1 ? gn.gz : gc.gz;
        const float kap = __fadd_rn(__fadd_rn(half_diff(nxr, nxl), half_diff(nyr, nyl)), half_diff(nzr, nzl));
        const float lap = __fadd_rn(__fadd_rn(half_diff(gxr, gxl), half_diff(gyr, gyl)), half_diff(gzr, gzl));
        const float dh = dirac<A>(p0, c.eps);
        const float out = update_phi(p0, dh, S.DT[C], kap, lap, c.dt, c.nu, c.mu);
        const size_t vi = (size_t)sc * k.WH + k.col;
        k.phi_out[vi] = out;
        if (!isfinite(out)) atomicOr(flag, kFlagNonFinite);
        if constexpr (DEBUG) {
            const bool inside = k.inside_xy && sc >= k.r && sc < k.L - k.r;
            if (!inside) {
                dbg.f[0 * dbg.n + vi] = 1.0f;
                dbg.f[1 * dbg.n + vi] = 1.0f;
                if (!c.full_data) {  // else the data-term kernels wrote e everywhere
                    const float I = load_img(k.s->img, vi, c.img_f32);
                    const float d = __fsub_rn(I, 1.0f);
                    dbg.f[2 * dbg.n + vi] = __fmul_rn(d, d);
                    dbg.f[3 * dbg.n + vi] = __fmul_rn(d, d);
                }
            }
            dbg.f[4 * dbg.n + vi] = dh;
            dbg.f[5 * dbg.n + vi] = kap;
            dbg.f[6 * dbg.n + vi] = lap;
            dbg.f[7 * dbg.n + vi] = grad_mag(gc.gx, Gb[C][k.w][k.lane].y, gc.gz);
        }
    }
    S.P[C] = p3;    // plane rel+3
    S.EX[C] = exn;  // plane rel+3
    S.EY[C] = eyn;
    S.DT[C1] = dn;  // plane rel+1
}

// Border-band data factor (f_out = f_in = 30/30 = 1) from the image at ip.
__device__ __forceinline__ float border_data(const unsigned char *ip, const StepConst &c) {
    const float I = c.img_f32 ? __ldg(reinterpret_cast<const float *>(ip)) : (float)__ldg(ip);
    const float d = __fsub_rn(I, 1.0f);
    const float e = __fmul_rn(d, d);
    return data_factor(e, e, c.l1, c.l2, c.lam_equal != 0);
}

// Fast step: the same arithmetic as stencil_step with every boundary rule
// that depends on the thread's voxel decided once per thread (rows of the
// y neighbours in the shared rings, x face flags) and phi, the output, the
// data factor and the image read through pointers that advance one plane per
// step.  The two extra rows of Pb hold the y neighbours of the halo rows.
// In the reference boundary mode, lane 0 of a block at x = 0 carries the
// previous linear element of lane 1's voxel, (W - 1, y - 1): its phi and its
// normalised gradient reach lane 1 through the ordinary shuffles.
// INSIDE: every output of the block lies in the valid region (blk_inside).
// EDGE: the step may meet a z rule or an end of the block's plane range
// (steps of the first and last groups of three, and groups near the first or
// last plane of the volume); otherwise every plane test is known to pass.
// FACE: the block touches an x or y face (per-thread rules apply).
// acc collects out * 0, which is NaN once any output is not finite.
template <int C, Arith A, bool INSIDE, bool EDGE, bool FACE>
__device__ __forceinline__ void stencil_step_f(const StencilCtx &k, const StepConst &c, StencilState &S, int sc,
                                               const float *&pp, float *&op, const float *&dp,
                                               const unsigned char *&ip, float (*Pb)[ST_WARPS + 2][32],
                                               float2 (*Gb)[ST_WARPS][32], float &acc) {
    constexpr int C1 = (C + 1) % 3, C2 = (C + 2) % 3;
    float p3 = 0.0f, exn = 0.0f, eyn = 0.0f;  // plane sc + 3
    if (!EDGE || sc + 3 < k.L) {
        if (!FACE || k.in) p3 = __ldg(pp);
        if (k.need_x) exn = __ldg(pp + k.xoff);
        if (k.need_y) eyn = __ldg(pp + k.yoff);
    }
    float dn = 0.0f;  // data factor of plane sc + 1
    const int pd = sc + 1;
    if (k.outp && (!EDGE || (pd >= k.z0 && pd < k.z1))) {
        if (INSIDE || (k.inside_xy && pd >= k.r && pd < k.L - k.r)) dn = __ldg(dp);
        else dn = border_data(ip, c);
    }
    dp += k.dplane;
    if (!INSIDE) ip += k.WH * (c.img_f32 ? 4 : 1);
    pp += k.WH;
    Pb[C2][k.w + 1][k.lane] = S.P[C2];
    if (k.w == 0) Pb[C2][0][k.lane] = S.EY[C2];
    if (k.w == ST_WARPS - 1) Pb[C2][ST_WARPS + 1][k.lane] = S.EY[C2];
    const float p0 = S.P[C], p1 = S.P[C1], p2 = S.P[C2];
    float L1 = __shfl_up_sync(0xffffffffu, p1, 1);
    float R1 = __shfl_down_sync(0xffffffffu, p1, 1);
    if (k.lane == 0) L1 = S.EX[C1];
    if (k.lane == 31) R1 = S.EX[C1];
    if (FACE) {
        if (k.xl_self) L1 = p1;
        if (k.xr_self) R1 = p1;
    }
    const float U1 = Pb[C1][k.urow][k.lane];
    const float D1 = Pb[C1][k.drow][k.lane];
    // gradient of plane pn = sc + 1 (z rules at the first and last plane; a
    // plane outside the volume gets a value that no output reads)
    const int pn = sc + 1;
    const GN gn = gn_from<A>(L1, R1, U1, D1, (!EDGE || pn > 0) ? p0 : p1, (!EDGE || pn < k.L - 1) ? p2 : p1);
    S.G[C1] = GN4{gn.nx, gn.gx, gn.nz, gn.gz};
    Gb[C1][k.w][k.lane] = make_float2(gn.ny, gn.gy);
    __syncthreads();
    const GN4 &gc = S.G[C];
    float nxL = __shfl_up_sync(0xffffffffu, gc.nx, 1), nxR = __shfl_down_sync(0xffffffffu, gc.nx, 1);
    float gxL = __shfl_up_sync(0xffffffffu, gc.gx, 1), gxR = __shfl_down_sync(0xffffffffu, gc.gx, 1);
    if ((!EDGE || sc >= k.z0) && k.outp) {
        if (FACE) {
            if (k.xl_self) {
                nxL = gc.nx;
                gxL = gc.gx;
            }
            if (k.xr_self) {
                nxR = gc.nx;
                gxR = gc.gx;
            }
        }
        const float2 yl2 = Gb[C][k.gwl][k.lane], yr2 = Gb[C][k.gwr][k.lane];
        const float nyl = yl2.x, nyr = yr2.x, gyl = yl2.y, gyr = yr2.y;
        const GN4 &gp = S.G[C2];
        const bool zlo = !EDGE || sc > 0, zhi = !EDGE || sc < k.L - 1;
        const float nzl = zlo ? gp.nz : gc.nz, nzr = zhi ? gn.nz : gc.nz;
        const float gzl = zlo ? gp.gz : gc.gz, gzr = zhi ? gn.gz : gc.gz;
        const float kap = __fadd_rn(__fadd_rn(half_diff(nxR, nxL), half_diff(nyr, nyl)), half_diff(nzr, nzl));
        const float lap = __fadd_rn(__fadd_rn(half_diff(gxR, gxL), half_diff(gyr, gyl)), half_diff(gzr, gzl));
        const float dh = dirac<A>(p0, c.eps);
        const float out = update_phi(p0, dh, S.DT[C], kap, lap, c.dt, c.nu, c.mu);
        *op = out;
        acc = __fmaf_rn(out, 0.0f, acc);
    }
    op += k.WH;
    S.P[C] = p3;
    S.EX[C] = exn;
    S.EY[C] = eyn;
    S.DT[C1] = dn;
}

// The steps of a block on the fast path in groups of three (one per ring
// slot); groups that can meet no z rule and no end of the plane range run
// without the plane tests.
template <Arith A, bool INSIDE, bool FACE>
__device__ __forceinline__ void stencil_planes_f(const StencilCtx &k, const StepConst &c, StencilState &S, int count,
                                                 const float *&pp, float *&op, const float *&dp,
                                                 const unsigned char *&ip, float (*Pb)[ST_WARPS + 2][32],
                                                 float2 (*Gb)[ST_WARPS][32], float &acc) {
    for (int i = 0; i < count; i += 3) {
        const int sc = k.first + i;
        const bool edge = i == 0 || i + 3 >= count || sc <= 0 || sc + 5 >= k.L;
        if (edge) {
            stencil_step_f<0, A, INSIDE, true, FACE>(k, c, S, sc, pp, op, dp, ip, Pb, Gb, acc);
            if (i + 1 < count) stencil_step_f<1, A, INSIDE, true, FACE>(k, c, S, sc + 1, pp, op, dp, ip, Pb, Gb, acc);
            if (i + 2 < count) stencil_step_f<2, A, INSIDE, true, FACE>(k, c, S, sc + 2, pp, op, dp, ip, Pb, Gb, acc);
        } else {
            stencil_step_f<0, A, INSIDE, false, FACE>(k, c, S, sc, pp, op, dp, ip, Pb, Gb, acc);
            stencil_step_f<1, A, INSIDE, false, FACE>(k, c, S, sc + 1, pp, op, dp, ip, Pb, Gb, acc);
            stencil_step_f<2, A, INSIDE, false, FACE>(k, c, S, sc + 2, pp, op, dp, ip, Pb, Gb, acc);
        }
    }
}

// ---------------------------------------------------------------------------
// Box e-term, CUDA_RSF/kernel.cu:25-55 with s = (int)sigma2 >= 1: for every
// voxel c, e = sum over the neighbours n of the (2s+1)^3 box that lie inside
// the volume of w (I_n - f(c))^2, w = 1/(2s+1)^2, accumulated in the
// reference's order (y outer, then x, then z) with each term fused in double
// and rounded to float.  f(c) comes from the z-pass in the valid region and
// is 30/30 = 1 in the border band.  Writes the data factor of every voxel;
// runs on the stencil's tiling (lanes 1..30 x warps 1..14 x 32 planes).
// ---------------------------------------------------------------------------
template <bool DEBUG>
__global__ void __launch_bounds__(ST_WARPS * 32) box_kernel(const SubVolDev *__restrict__ svs,
                                                            const int *__restrict__ pre, const StepConst c,
                                                            DebugOut dbg) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev &s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int ntx = (s.W + ST_OX - 1) / ST_OX, nty = (s.H + ST_OY - 1) / ST_OY;
    const int tx = t % ntx;
    t /= ntx;
    const int ty = t % nty;
    const int tz = t / nty;
    const int x = tx * ST_OX - 1 + lane, y = ty * ST_OY - 1 + w;
    if (lane < 1 || lane > ST_OX || w < 1 || w > ST_OY || x >= s.W || y >= s.H) return;
    const int z0 = tz * c.zc, z1 = min(z0 + c.zc, s.L);
    const int bs = c.box, r = c.r;
    const double wt = 1.0 / (double)((2 * bs + 1) * (2 * bs + 1));
    const size_t WH = (size_t)s.W * s.H, nvalid = (size_t)s.Wp * s.Hv * s.Lv;
    float *dfull = s.db + 2 * nvalid;
    const bool valid_xy = s.Wv > 0 && x >= r && x < r + s.Wv && y >= r && y < r + s.Hv;
    for (int z = z0; z < z1; ++z) {
        float fo = 1.0f, fi = 1.0f;
        if (valid_xy && z >= r && z < r + s.Lv) {
            const size_t di = ((size_t)(z - r) * s.Hv + (y - r)) * s.Wp + (x - r);
            fo = s.db[di];
            fi = s.db[nvalid + di];
        }
        float s1 = 0.0f, s2 = 0.0f;
        for (int u = -bs; u <= bs; ++u) {
            const int yy = y + u;
            if (yy < 0 || yy >= s.H) continue;
            for (int v = -bs; v <= bs; ++v) {
                const int xx = x + v;
                if (xx < 0 || xx >= s.W) continue;
                for (int q = -bs; q <= bs; ++q) {
                    const int zz = z + q;
                    if (zz < 0 || zz >= s.L) continue;
                    const float In = load_img(s.img, (size_t)zz * WH + (size_t)yy * s.W + xx, c.img_f32);
                    const float d1 = __fsub_rn(In, fo), d2 = __fsub_rn(In, fi);
                    s1 = __double2float_rn(__fma_rn(__dmul_rn(wt, (double)d1), (double)d1, (double)s1));
                    s2 = __double2float_rn(__fma_rn(__dmul_rn(wt, (double)d2), (double)d2, (double)s2));
                }
            }
        }
        const size_t vi = (size_t)z * WH + (size_t)y * s.W + x;
        dfull[vi] = data_factor(s1, s2, c.l1, c.l2, c.lam_equal != 0);
        if (DEBUG) {
            dbg.f[2 * dbg.n + vi] = s1;
            dbg.f[3 * dbg.n + vi] = s2;
        }
    }
}

template <Arith A, bool DEBUG>
__global__ void __launch_bounds__(ST_WARPS * 32, 2) stencil_kernel(const SubVolDev *__restrict__ svs,
                                                                   const int *__restrict__ pre,
                                                                   const StepConst c, int parity,
                                                                   unsigned *__restrict__ flag, DebugOut dbg) {
    __shared__ float Pb[3][ST_WARPS + 2][32];
    __shared__ float2 Gb[3][ST_WARPS][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev &s = svs[sv];
    int t = b - __ldg(pre + sv);
    StencilCtx k;
    k.s = &s;
    k.W = s.W;
    k.H = s.H;
    k.L = s.L;
    k.r = c.r;
    const int ntx = (k.W + ST_OX - 1) / ST_OX, nty = (k.H + ST_OY - 1) / ST_OY;
    const int tx = t % ntx;
    t /= ntx;
    const int ty = t % nty;
    const int tz = t / nty;
    const int x0 = tx * ST_OX, y0 = ty * ST_OY;
    k.ref = c.boundary == 0;
    // Every block takes the fast path but in the debug step and, in the
    // reference mode, the blocks at x = 0 that hold row 0 (where the previous
    // linear element of voxel (0, 0) lies in the previous plane).
    const bool fast = !DEBUG && !(k.ref && x0 == 0 && y0 < 2);
    const bool prev_lane = fast && k.ref && x0 == 0 && lane == 0;
    k.x = x0 - 1 + lane;
    k.y = y0 - 1 + w;
    k.w = w;
    k.lane = lane;
    k.z0 = tz * c.zc;
    k.z1 = min(k.z0 + c.zc, k.L);
    k.first = k.z0 - 2;
    // the thread's voxel: lane 0 at x = 0 may carry (W - 1, y - 1)
    const int ex = prev_lane ? k.W - 1 : k.x, ey = prev_lane ? k.y - 1 : k.y;
    k.in = ex >= 0 && ex < k.W && ey >= 0 && ey < k.H;
    k.outp = k.in && !prev_lane && lane >= 1 && lane <= ST_OX && w >= 1 && w <= ST_OY;
    k.WH = (size_t)k.W * k.H;
    k.col = k.in ? (size_t)ey * k.W + ex : 0;
    k.phi = (parity ? s.phi[1] : s.phi[0]) + k.col;
    k.phi_out = parity ? s.phi[0] : s.phi[1];
    const bool valid = s.Wv > 0;
    const int r = k.r;
    k.inside_xy = valid && ex >= r && ex < k.W - r && ey >= r && ey < k.H - r;
    k.blk_inside = valid && x0 >= r && x0 + ST_OX - 1 < k.W - r && y0 >= r && y0 + ST_OY - 1 < k.H - r &&
                   k.z0 >= r && k.z1 - 1 < k.L - r;
    k.dplane = (size_t)s.Wp * s.Hv;
    k.dcol = k.inside_xy ? s.db + (size_t)(ey - r) * s.Wp + (ex - r) : s.db;
    if (c.full_data) {  // every voxel's data factor comes from the box or expanded data-term kernels
        k.blk_inside = true;
        k.dplane = k.WH;
        k.dcol = s.db + 2 * (size_t)s.Wp * s.Hv * s.Lv + k.col + (size_t)r * k.WH;
    }
    // The shuffles and shared rows supply every neighbour except: x-1 for
    // lane 0 (and, on the debug path, the previous linear element for x == 0
    // in the reference mode), both at linear offset -1; x+1 for lane 31;
    // y-1 / y+1 for the halo rows.  Corner threads of the halo are never read.
    const bool halo_row = w == 0 || w == ST_WARPS - 1;
    const bool halo_col = lane == 0 || lane == 31;
    k.need_x = k.in && !(halo_row && halo_col) &&
               ((lane == 0) || (!fast && k.x == 0 && k.ref) || (lane == 31 && ex + 1 < k.W));
    k.xoff = lane == 31 ? 1 : -1;
    k.need_y = k.in && halo_row && !halo_col && (w == 0 ? ey > 0 : ey + 1 < k.H);
    k.yoff = w == 0 ? -(ptrdiff_t)k.W : (ptrdiff_t)k.W;
    k.xl_self = !k.ref && ex == 0;
    k.xr_self = ex == k.W - 1;
    k.urow = ey > 0 ? w : w + 1;
    k.drow = ey < k.H - 1 ? w + 2 : w + 1;
    k.gwl = ey > 0 ? w - 1 : w;
    k.gwr = ey < k.H - 1 ? w + 1 : w;

    StencilState S;
    const int sp = k.first;
    S.P[0] = st_ld(k, sp);
    S.P[1] = st_ld(k, sp + 1);
    S.P[2] = st_ld(k, sp + 2);
    S.EX[1] = st_ldx(k, sp + 1);
    S.EY[1] = st_ldy(k, sp + 1);
    S.EX[2] = st_ldx(k, sp + 2);
    S.EY[2] = st_ldy(k, sp + 2);
    S.EX[0] = S.EY[0] = 0.0f;
    S.DT[0] = S.DT[1] = S.DT[2] = 0.0f;
    for (int i = 0; i < 3; ++i) S.G[i] = GN4{0.f, 0.f, 0.f, 0.f};
    Pb[1][w + 1][lane] = S.P[1];
    if (w == 0) Pb[1][0][lane] = S.EY[1];
    if (w == ST_WARPS - 1) Pb[1][ST_WARPS + 1][lane] = S.EY[1];
    __syncthreads();
    const int count = k.z1 - k.first;
    if (fast) {
        const float *pp = k.phi + (ptrdiff_t)(k.first + 3) * (ptrdiff_t)k.WH;
        float *op = k.phi_out + (ptrdiff_t)k.first * (ptrdiff_t)k.WH + (ptrdiff_t)k.col;
        // plane first + 1 of the data column and of the image (read only
        // from plane z0 on)
        const float *dp = k.dcol + ((ptrdiff_t)k.first + 1 - k.r) * (ptrdiff_t)k.dplane;
        const ptrdiff_t esz = c.img_f32 ? 4 : 1;
        const unsigned char *ip = static_cast<const unsigned char *>(s.img) +
                                  ((ptrdiff_t)k.col + ((ptrdiff_t)k.first + 1) * (ptrdiff_t)k.WH) * esz;
        // x/y-interior blocks: every thread and neighbour load inside, no x
        // or y face rule
        const bool face = !(x0 >= 2 && x0 + 32 <= k.W && y0 >= 2 && y0 + ST_OY + 2 <= k.H);
        float acc = 0.0f;
        if (face) {
            if (k.blk_inside) stencil_planes_f<A, true, true>(k, c, S, count, pp, op, dp, ip, Pb, Gb, acc);
            else stencil_planes_f<A, false, true>(k, c, S, count, pp, op, dp, ip, Pb, Gb, acc);
        } else {
            if (k.blk_inside) stencil_planes_f<A, true, false>(k, c, S, count, pp, op, dp, ip, Pb, Gb, acc);
            else stencil_planes_f<A, false, false>(k, c, S, count, pp, op, dp, ip, Pb, Gb, acc);
        }
        if (!isfinite(acc)) atomicOr(flag, kFlagNonFinite);
        return;
    }
    for (int i = 0; i < count; i += 3) {
        stencil_step<0, A, DEBUG>(k, c, S, i, Pb, Gb, flag, dbg);
        if (i + 1 < count) stencil_step<1, A, DEBUG>(k, c, S, i + 1, Pb, Gb, flag, dbg);
        if (i + 2 < count) stencil_step<2, A, DEBUG>(k, c, S, i + 2, Pb, Gb, flag, dbg);
    }
}

}  // namespace rsf
