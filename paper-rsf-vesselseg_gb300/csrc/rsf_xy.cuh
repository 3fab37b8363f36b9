// rsf_xy.cuh -- fused x/y-pass: H, 1-H, I H, I (1-H) (kernel.cu:210-298),
// their valid correlation along x (kernel.cu:1000-1014) and along y
// (kernel.cu:1017-1031) in one kernel, for the tap counts that are a
// multiple of XY_R (21 and 35).
//
// A block owns TX x-outputs (a multiple of XY_R, chosen per launch) of one z
// plane and streams y in chunks of XY_R rows.  Per chunk:
//   A0  each thread forms the four fields of up to 5 input elements (rows of
//       the chunk x TX + k - 1 columns) from phi and I it loaded during the
//       previous chunk, into two shared pair planes (H, 1-H) and
//       (I H, I (1-H)) of float2;
//   A1  each thread correlates XY_R consecutive x-outputs of one row and one
//       pair (packed f32x2 multiply-adds over ascending taps from +0) into a
//       shared row buffer;
//   B   each thread takes one column of one pair and adds the chunk's rows
//       into k rotating accumulators (the accumulator of y-output o is slot
//       o mod k; a chunk of XY_R rows starts at a multiple of XY_R, so every
//       slot index is a constant of the unrolled code), writing each y-output
//       as soon as its k-th row has been added.
// The x fields never reach global memory; the y fields are written once, as
// float2 pairs: pair 0 (H, 1-H) and pair 1 (I H, I (1-H)), each Wp x Hv x L.
// Summation order per output is the reference's (x taps ascending, then y
// taps ascending), so the results equal the separate passes bit for bit.
#pragma once
#include "rsf_kernels.cuh"

namespace rsf {

__host__ __device__ inline size_t xy_smem_bytes(int tx, int k) {
    const int span = tx + k - 1;
    return sizeof(float2) * ((size_t)2 * XY_R * span + (size_t)XY_R * 2 * tx);
}

// XB consecutive valid x-correlations of one pair plane (stride-1 float2).
template <int K, int XB>
__device__ __forceinline__ void xconv_plane(const float2 *src, const StepConst &c, float2 (&acc)[XB]) {
#pragma unroll
    for (int q = 0; q < XB + K - 1; ++q) {
        const float2 v = src[q];
#pragma unroll
        for (int m = 0; m < XB; ++m) {
            const int tt = q - m;
            if (tt == 0) acc[m] = fma2(v, c.taps2[0], make_float2(0.f, 0.f));
            else if (tt > 0 && tt < K) acc[m] = fma2(v, c.taps2[tt], acc[m]);
        }
    }
}

// Rows CC*XY_R .. CC*XY_R + XY_R - 1 (mod K) of the y stream of one column.
template <int K, int CC>
__device__ __forceinline__ void ystream_chunk(const float2 *bsrc, int row_stride, float2 (&acc)[K], const StepConst &c,
                                              int y0, int Hv, bool live, float2 *out, size_t wp) {
#pragma unroll
    for (int jj = 0; jj < XY_R; ++jj) {
        constexpr int base = CC * XY_R;
        const float2 v = bsrc[jj * row_stride];
#pragma unroll
        for (int tt = 0; tt < K; ++tt) {
            const int slot = (base + jj - tt + K) % K;
            if (tt == 0) acc[slot] = fma2(v, c.taps2[0], make_float2(0.f, 0.f));
            else acc[slot] = fma2(v, c.taps2[tt], acc[slot]);
        }
        const int o = y0 + jj - (K - 1);
        if (live && o >= 0 && o < Hv) out[(size_t)o * wp] = acc[(base + jj + 1) % K];
    }
}

template <int K, int CC = 0>
__device__ __forceinline__ void ystream_dispatch(int cc, const float2 *bsrc, int row_stride, float2 (&acc)[K],
                                                 const StepConst &c, int y0, int Hv, bool live, float2 *out,
                                                 size_t wp) {
    if constexpr (CC < K / XY_R) {
        if (cc == CC) {
            ystream_chunk<K, CC>(bsrc, row_stride, acc, c, y0, Hv, live, out, wp);
            return;
        }
        ystream_dispatch<K, CC + 1>(cc, bsrc, row_stride, acc, c, y0, Hv, live, out, wp);
    }
}

// Two resident blocks per SM for 21 taps; the 35 rotating accumulator pairs
// of 35 taps need the registers of one block per SM.
template <int K>
__global__ void __launch_bounds__(2 * XY_TX_MAX, K <= 21 ? 2 : 1) xypass_kernel(const SubVolDev *__restrict__ svs,
                                                                   const int *__restrict__ pre, const StepConst c,
                                                                   int parity) {
    static_assert(K % XY_R == 0, "the row chunk must divide the tap count");
    constexpr int R = XY_R, XB = XY_R;
    constexpr int NE = 5;  // elements per thread per chunk: ceil(R (TX + K - 1) / (2 TX)) <= 5 for TX >= 84
    extern __shared__ float2 xsm[];
    const int TX = c.xy_tx, NG = TX / XB, span = TX + K - 1, NT = 2 * TX;
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    const int t = b - __ldg(pre + sv);
    const int ntx = (s.Wv + TX - 1) / TX;
    const int tx = t % ntx, z = t / ntx;
    const int x0 = tx * TX;
    const int tid = threadIdx.x;
    float2 *hp = xsm;                 // [2][R][span]
    float2 *xo = xsm + 2 * R * span;  // [R][2][TX]
    const size_t plane = (size_t)z * s.H * s.W;
    const float *phi = (parity ? s.phi[1] : s.phi[0]) + plane;
    const unsigned char *img8 = static_cast<const unsigned char *>(s.img) + plane;
    const float *imgf = static_cast<const float *>(s.img) + plane;

    // A0: this thread's elements are tid + q NT of the chunk's R x span block;
    // NT = span + de with de = TX - K + 1 >= 0, so each step is one row down
    // and de columns right.
    const int e0 = tid % span, j0 = tid / span, de = NT - span;
    float pv[NE], iv[NE];
    auto load_chunk = [&](int y0) {
        int e = e0, j = j0;
#pragma unroll
        for (int q = 0; q < NE; ++q) {
            const int y = y0 + j, x = x0 + e;
            const bool ok = j < R && y < s.H && x < s.W;
            const size_t off = (size_t)y * s.W + x;
            pv[q] = ok ? __ldg(phi + off) : 0.0f;
            iv[q] = ok ? (c.img_f32 ? __ldg(imgf + off) : (float)__ldg(img8 + off)) : 0.0f;
            e += de;
            j += 1;
            if (e >= span) {
                e -= span;
                j += 1;
            }
        }
    };
    auto fields_chunk = [&](int y0) {
        int e = e0, j = j0;
#pragma unroll
        for (int q = 0; q < NE; ++q) {
            if (j < R) {
                float2 a = make_float2(0.f, 0.f), m = a;
                if (y0 + j < s.H && x0 + e < s.W) {
                    const float h = heaviside<Arith::Portable>(pv[q], c.eps);
                    const float hi = __fsub_rn(1.0f, h);
                    a = make_float2(h, hi);
                    m = make_float2(__fmul_rn(iv[q], h), __fmul_rn(iv[q], hi));
                }
                hp[j * span + e] = a;
                hp[(R + j) * span + e] = m;
            }
            e += de;
            j += 1;
            if (e >= span) {
                e -= span;
                j += 1;
            }
        }
    };

    // A1: row ja, pair pa, x-group g (XB outputs); NT = 2 R NG tasks.
    const int jpa = tid / NG, g = tid - jpa * NG;
    const int ja = jpa >> 1, pa = jpa & 1;
    const float2 *asrc = hp + (pa * R + ja) * span + g * XB;
    float2 *adst = xo + (ja * 2 + pa) * TX + g * XB;

    // B: one column of one pair.
    const int pb = tid >= TX ? 1 : 0, col = tid - pb * TX;
    const bool live = x0 + col < s.Wv;
    const float2 *bsrc = xo + pb * TX + col;
    float2 *out = reinterpret_cast<float2 *>(s.yb) + (size_t)pb * s.Wp * s.Hv * s.L + (size_t)z * s.Hv * s.Wp + x0 + col;
    float2 acc[K];
#pragma unroll
    for (int q = 0; q < K; ++q) acc[q] = make_float2(0.f, 0.f);

    const int nchunks = (s.H + R - 1) / R;
    load_chunk(0);
    for (int ch = 0; ch < nchunks; ++ch) {
        const int y0 = ch * R;
        fields_chunk(y0);
        if (ch + 1 < nchunks) load_chunk(y0 + R);
        __syncthreads();
        {
            float2 xa[XB];
            xconv_plane<K, XB>(asrc, c, xa);
#pragma unroll
            for (int m = 0; m < XB; ++m) adst[m] = xa[m];
        }
        __syncthreads();
        ystream_dispatch<K>(ch % (K / R), bsrc, 2 * TX, acc, c, y0, s.Hv, live, out, (size_t)s.Wp);
    }
}

}  // namespace rsf
