// rsf_zt.cuh -- z-pass over the fused x/y-pass output: valid correlation
// along z (kernel.cu:1035-1049), local fits f = blur(I H)/blur(H)
// (kernel.cu:191-207), e = (I - f)^2 (kernel.cu:25-55 with sigma2 = 0) and
// the data factor lambda (e_out - e_in) of the valid region.
//
// A block owns a tile of ZT_X x ZT_Y columns and streams z.  One producer
// warp moves each z plane of the tile's two pair planes into a ring of ZT_D
// shared-memory slots with one TMA tile load (cp.async.bulk.tensor, 4-D box
// {2 ZT_X floats, ZT_Y rows, 1 plane, 2 pairs} of the pair planes, completed
// on the slot's "full" mbarrier); eight consumer warps take one column and
// one pair per thread, add each plane into k rotating accumulator pairs (the
// accumulator of z-output o is slot o mod k, a constant of the k-unrolled
// code), release the slot on its "empty" mbarrier and, when output o is
// complete, form the fits with the partner thread of the other pair (lane
// xor 16) and write lambda (e_out - e_in).
#pragma once
#include "rsf_kernels.cuh"
#include "rsf_tma.cuh"

namespace rsf {

constexpr int ZT_X = 32;                                     // columns per tile
constexpr int ZT_Y = 4;                                      // rows per tile
constexpr int ZT_D = 8;                                      // ring slots (planes in flight)
constexpr int ZT_CONSUMERS = ZT_X * ZT_Y * 2 / 32;           // consumer warps
constexpr int ZT_THREADS = (ZT_CONSUMERS + 1) * 32;          // + the producer warp
constexpr unsigned ZT_SLOT_BYTES = 2u * ZT_Y * 2 * ZT_X * 4;  // bytes of one plane box

struct ZtShared {
    alignas(128) float slot[ZT_D][2][ZT_Y][2 * ZT_X];  // [slot][pair][row][x as float2]
    uint64_t full[ZT_D];
    uint64_t empty[ZT_D];
};

template <int K>
__global__ void __launch_bounds__(ZT_THREADS, K <= 21 ? 2 : 1) ztpass_kernel(const SubVolDev *__restrict__ svs,
                                                              const int *__restrict__ pre, const StepConst c,
                                                              unsigned *__restrict__ flag) {
    __shared__ ZtShared sh;
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev &s = svs[sv];
    const int t = b - __ldg(pre + sv);
    const int Wv = s.Wv, Hv = s.Hv, L = s.L;
    const int ntx = (Wv + ZT_X - 1) / ZT_X;
    const int x0 = (t % ntx) * ZT_X, y0 = (t / ntx) * ZT_Y;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const void *map = static_cast<const unsigned char *>(c.ymaps) + (size_t)sv * TMAP_BYTES;
    if (threadIdx.x == 0) {
        for (int q = 0; q < ZT_D; ++q) {
            mbar_init(&sh.full[q], 1);
            mbar_init(&sh.empty[q], ZT_CONSUMERS);
        }
        fence_barrier_init();
    }
    __syncthreads();
    if (warp == ZT_CONSUMERS) {
        // producer: plane i into slot i mod ZT_D once the consumers have
        // released the plane ZT_D before it
        if (lane == 0) {
            tensormap_acquire(map);
            for (int i = 0; i < L; ++i) {
                const int q = i % ZT_D;
                if (i >= ZT_D && !mbar_wait(&sh.empty[q], (unsigned)((i / ZT_D) - 1) & 1u)) {
                    atomicOr(flag, kFlagTimeout);
                    break;
                }
                mbar_arrive_expect_tx(&sh.full[q], ZT_SLOT_BYTES);
                tma_load_4d(&sh.slot[q][0][0][0], map, 2 * x0, y0, i, 0, &sh.full[q]);
            }
        }
        return;
    }
    // consumer: column x, pair p (lanes 0-15 pair 0, 16-31 pair 1)
    const int yy = warp >> 1, xx = (warp & 1) * 16 + (lane & 15), p = lane >> 4;
    const int x = x0 + xx, y = y0 + yy;
    const bool act = x < Wv && y < Hv;
    const int r = c.r;
    const size_t img_plane = (size_t)s.W * s.H;
    const size_t img_off = ((size_t)r * s.H + (size_t)(y + r)) * s.W + (size_t)(x + r);
    const unsigned char *im8 = static_cast<const unsigned char *>(s.img) + img_off;
    const float *imf = static_cast<const float *>(s.img) + img_off;
    float *dbp = s.db + (size_t)y * s.Wp + x;
    const size_t db_plane = (size_t)s.Wp * Hv;
    int sl = 0;
    unsigned ph = 0;
    bool ok = true;
    float2 acc[K];
#pragma unroll
    for (int q = 0; q < K; ++q) acc[q] = make_float2(0.f, 0.f);
    // K planes with compile-time accumulator slots (plane base + j is slot j)
    auto block = [&](int base, bool guard) {
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const int i = base + j;
            if (guard && i >= L) break;
            const int o = i - (K - 1);
            // the image at this column's voxel of output plane o, issued early
            float I = 0.0f;
            if (o >= 0 && act) I = c.img_f32 ? __ldg(imf + (size_t)o * img_plane) : (float)__ldg(im8 + (size_t)o * img_plane);
            if (ok && !mbar_wait(&sh.full[sl], ph)) {
                ok = false;
                atomicOr(flag, kFlagTimeout);
            }
            const float2 v = *reinterpret_cast<const float2 *>(&sh.slot[sl][p][yy][2 * xx]);
            __syncwarp();
            if (lane == 0) mbar_arrive(&sh.empty[sl]);
            if (++sl == ZT_D) {
                sl = 0;
                ph ^= 1u;
            }
#pragma unroll
            for (int tt = 0; tt < K; ++tt) {
                const int q = (j - tt + K) % K;
                if (tt == 0) acc[q] = fma2(v, c.taps2[0], make_float2(0.f, 0.f));
                else acc[q] = fma2(v, c.taps2[tt], acc[q]);
            }
            if (o >= 0) {
                // pair 0 holds (H, 1-H), pair 1 (I H, I (1-H)) of the same column
                const float2 B = acc[(j + 1) % K];
                const float other = __shfl_xor_sync(0xffffffffu, p ? B.x : B.y, 16);
                const float num = p ? B.y : other, den = p ? other : B.x;
                const float fv = __fdiv_rn(num, den);  // pair 0: f_out, pair 1: f_in
                const float d = __fsub_rn(I, fv);
                const float e = __fmul_rn(d, d);
                const float e_in = __shfl_xor_sync(0xffffffffu, e, 16);
                if (p == 0 && act) dbp[(size_t)o * db_plane] = data_factor(e, e_in, c.l1, c.l2, c.lam_equal != 0);
            }
        }
    };
    int base = 0;
    for (; base + K <= L; base += K) block(base, false);
    if (base < L) block(base, true);
}

}  // namespace rsf
