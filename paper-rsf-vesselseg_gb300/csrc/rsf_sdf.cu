// rsf_sdf.cu -- the initial level set: the exact signed Euclidean distance of
// a seed region, on the device.
//
// The reference builds phi0 on the host: it subtracts 13 from the seed volume
// and calls tiralib's volume::sdf() (CUDA_RSF/main.cpp:174-183).  tiralib is
// not part of the reference checkout, so the transform is defined here on its
// own terms: a voxel is inside when seed > threshold; phi0 is +d(p, outside)
// at inside voxels and -d(p, inside) at outside voxels, d the Euclidean
// distance in voxels between voxel centres.  When one class is empty the
// other gets +-(W + H + L), larger than any distance in the box.
//
// Each class is one exact distance transform, computed separably on squared
// integer distances (Felzenszwalb & Huttenlocher, "Distance Transforms of
// Sampled Functions", Theory of Computing 8, 2012):
//   rows    (x) one warp per row: nearest feature to the left and right by
//               warp max/min scans, squared;
//   columns (y, then z) one thread per column: the lower envelope of the
//               parabolas (q - v)^2 + f(v), evaluated at every q.
// Envelope intersections are compared exactly in 64-bit integers, so the
// squared distances are exact and phi0 = sqrt of an integer, correctly rounded.
// Column threads are adjacent in x, so every access of a column step is
// coalesced across the warp; the envelope stacks live in device scratch laid
// out [k][column] for the same reason.
#include <cuda_runtime.h>

#include <climits>

#include "rsf_internal.h"

namespace rsf {
namespace {

constexpr unsigned kInf = 0xffffffffu;
constexpr int kRowWarps = 8;
constexpr int kColThreads = 128;

__device__ __forceinline__ bool is_inside(const void *seed, int f32, size_t i, float thr) {
    const float v = f32 ? static_cast<const float *>(seed)[i] : (float)static_cast<const unsigned char *>(seed)[i];
    return v > thr;
}

// Squared distance along x to the nearest feature of the row (kInf when the
// row has none).  Features are the voxels whose class equals feat_inside.
__global__ void __launch_bounds__(32 * kRowWarps) sdf_rows(const void *seed, int f32, float thr, int feat_inside,
                                                           unsigned *d, int W, long long rows) {
    const long long row = (long long)blockIdx.x * kRowWarps + threadIdx.x / 32;
    if (row >= rows) return;  // uniform per warp
    const int lane = threadIdx.x & 31;
    const size_t base = (size_t)row * W;
    int carry = -1;  // last feature at or left of the chunk start
    for (int x0 = 0; x0 < W; x0 += 32) {
        const int x = x0 + lane;
        const bool f = x < W && is_inside(seed, f32, base + x, thr) == (feat_inside != 0);
        int v = f ? x : -1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v = max(v, u);
        }
        v = max(v, carry);
        if (x < W) d[base + x] = (unsigned)v;
        carry = __shfl_sync(0xffffffffu, v, 31);
    }
    int rcarry = INT_MAX;  // first feature at or right of the chunk end
    for (int x0 = ((W - 1) / 32) * 32; x0 >= 0; x0 -= 32) {
        const int x = x0 + lane;
        const bool f = x < W && is_inside(seed, f32, base + x, thr) == (feat_inside != 0);
        int v = f ? x : INT_MAX;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_down_sync(0xffffffffu, v, o);
            if (lane + o < 32) v = min(v, u);
        }
        v = min(v, rcarry);
        if (x < W) {
            const int left = (int)d[base + x];
            long long best = -1;
            if (left >= 0) best = x - left;
            if (v != INT_MAX && (best < 0 || v - x < best)) best = v - x;
            d[base + x] = best < 0 ? kInf : (unsigned)(best * best);
        }
        rcarry = __shfl_sync(0xffffffffu, v, 0);
    }
}

struct ColArgs {
    unsigned *d;        // squared distances, transformed in place (not FINAL)
    unsigned *sv;       // envelope stack: sample positions, [k][column]
    unsigned *sf;       // envelope stack: sample values
    long long ncols;
    int W;              // columns are numbered c = a * W + x
    long long plane;    // element offset of a column: (c / W) * plane + c % W
    long long stride;   // element step along the column
    int n;              // column length
    // FINAL: write phi at the voxels of the evaluated class
    const void *seed;
    int f32;
    float thr;
    int feat_inside;
    float *phi;
    float fill;
};

template <bool FINAL>
__global__ void __launch_bounds__(kColThreads) sdf_cols(ColArgs a) {
    const long long c = (long long)blockIdx.x * kColThreads + threadIdx.x;
    if (c >= a.ncols) return;
    const size_t base = (size_t)(c / a.W) * (size_t)a.plane + (size_t)(c % a.W);
    const size_t nc = (size_t)a.ncols;
    // Lower envelope over the finite samples; the top two entries stay in
    // registers as (position, F = f + position^2).
    int top = -1;
    long long vt = 0, Ft = 0, vp = 0, Fp = 0;
    for (int q = 0; q < a.n; q++) {
        const unsigned f = a.d[base + (size_t)q * (size_t)a.stride];
        if (f == kInf) continue;
        const long long Fq = (long long)f + (long long)q * q;
        // the top parabola is hidden when the new one overtakes it no later
        // than it overtakes the one below it
        while (top >= 1 && (Fq - Ft) * (vt - vp) <= (Ft - Fp) * ((long long)q - vt)) {
            top--;
            vt = vp;
            Ft = Fp;
            if (top >= 1) {
                vp = a.sv[(size_t)(top - 1) * nc + c];
                Fp = (long long)a.sf[(size_t)(top - 1) * nc + c] + vp * vp;
            }
        }
        top++;
        a.sv[(size_t)top * nc + c] = (unsigned)q;
        a.sf[(size_t)top * nc + c] = f;
        vp = vt;
        Fp = Ft;
        vt = q;
        Ft = Fq;
    }
    int k = 0;
    long long v0 = 0, f0 = 0, v1 = 0, F1 = 0;
    if (top >= 0) {
        v0 = a.sv[c];
        f0 = a.sf[c];
    }
    if (top >= 1) {
        v1 = a.sv[nc + c];
        F1 = (long long)a.sf[nc + c] + v1 * v1;
    }
    for (int q = 0; q < a.n; q++) {
        // move right while the next parabola is lower at q
        while (k < top && F1 - (f0 + v0 * v0) < 2LL * q * (v1 - v0)) {
            k++;
            v0 = v1;
            f0 = F1 - v1 * v1;
            if (k < top) {
                v1 = a.sv[(size_t)(k + 1) * nc + c];
                F1 = (long long)a.sf[(size_t)(k + 1) * nc + c] + v1 * v1;
            }
        }
        const size_t idx = base + (size_t)q * (size_t)a.stride;
        const long long dq = q - v0;
        const unsigned D = top < 0 ? kInf : (unsigned)(dq * dq + f0);
        if (!FINAL) {
            a.d[idx] = D;
        } else if (is_inside(a.seed, a.f32, idx, a.thr) != (a.feat_inside != 0)) {
            const float mag = D == kInf ? a.fill : __fsqrt_rn(__uint2float_rn(D));
            a.phi[idx] = a.feat_inside ? -mag : mag;
        }
    }
}

}  // namespace

cudaError_t launch_signed_distance(const void *seed, int f32, float thr, float *phi, int W, int H, int L,
                                   unsigned *scratch, cudaStream_t st) {
    const size_t N = (size_t)W * H * L;
    unsigned *d = scratch, *sv = scratch + N, *sf = scratch + 2 * N;
    const long long rows = (long long)H * L;
    const float fill = (float)W + (float)H + (float)L;
    for (int feat_inside = 0; feat_inside < 2; feat_inside++) {
        sdf_rows<<<(unsigned)((rows + kRowWarps - 1) / kRowWarps), 32 * kRowWarps, 0, st>>>(seed, f32, thr,
                                                                                           feat_inside, d, W, rows);
        ColArgs a{d, sv, sf, (long long)W * L, W, (long long)W * H, W, H, seed, f32, thr, feat_inside, phi, fill};
        sdf_cols<false><<<(unsigned)((a.ncols + kColThreads - 1) / kColThreads), kColThreads, 0, st>>>(a);
        a.ncols = (long long)W * H;
        a.plane = W;
        a.stride = (long long)W * H;
        a.n = L;
        sdf_cols<true><<<(unsigned)((a.ncols + kColThreads - 1) / kColThreads), kColThreads, 0, st>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace rsf
