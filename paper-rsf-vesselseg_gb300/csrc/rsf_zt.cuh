// rsf_zt.cuh -- z-pass fed by TMA: valid correlation along z
// (kernel.cu:1035-1049), local fits f = blur(I H)/blur(H) (kernel.cu:191-207),
// e = (I - f)^2 (kernel.cu:25-55 with sigma2 = 0) and the data factor
// lambda (e_out - e_in) of the valid region, for 21 and 35 taps.
//
// Input: the y-pass output as two float2 pair planes, pair 0 (H, 1-H) and
// pair 1 (I H, I (1-H)), each Wp x Hv x L.  A block owns a tile of ZT_X x ZT_Y
// columns and streams z.  One producer thread moves z plane i of the tile's
// two pair planes into ring slot i mod k with one TMA tile load
// (cp.async.bulk.tensor, 4-D box {2 ZT_X floats, ZT_Y rows, 1 plane, 2 pairs}).
// The ring is handed over in groups of ZT_G consecutive planes: each group
// completes on one "full" mbarrier (the bytes of its ZT_G loads) and is
// released on one "empty" mbarrier, so a consumer waits and arrives once per
// ZT_G planes.  The producer refills a group's slots with the planes k later
// once the consumers have released it.  Eight consumer warps
// take one column and one pair per thread and add each plane into k rotating
// accumulator pairs; in the k-unrolled loop the ring slot, its barrier phase
// and the accumulator of z-output o (slot o mod k) are constants.  When
// output o completes, the thread forms one fit with the partner thread of the
// other pair (lane xor 16) and pair 0 writes lambda (e_out - e_in).  The
// image word of output o is loaded 3 (21 taps) or 5 (35 taps) outputs ahead
// into a register ring and converted only when used.
#pragma once
#include "rsf_kernels.cuh"
#include "rsf_tma.cuh"

namespace rsf {

constexpr int ZT_X = 32;                                      // columns per tile
constexpr int ZT_Y = 4;                                       // rows per tile
constexpr int ZT_CONSUMERS = ZT_X * ZT_Y * 2 / 32;            // consumer warps
constexpr int ZT_THREADS = (ZT_CONSUMERS + 1) * 32;           // + the producer warp
constexpr unsigned ZT_SLOT_BYTES = 2u * ZT_Y * 2 * ZT_X * 4;  // bytes of one plane box
constexpr int ZT_G = 7;                                       // planes per barrier group (divides k)

// Image prefetch depth in outputs: a divisor of k (3 for 21, 5 for 35).
__host__ __device__ constexpr int zt_img_ahead(int k) { return k % 3 == 0 ? 3 : 5; }

__host__ __device__ constexpr size_t zt_smem_bytes(int k) {
    return (size_t)k * ZT_SLOT_BYTES + 2 * (size_t)(k / ZT_G) * sizeof(uint64_t);
}

template <int K>
__global__ void __launch_bounds__(ZT_THREADS, K <= 21 ? 3 : 1) ztpass_kernel(const SubVolDev *__restrict__ svs,
                                                                            const int *__restrict__ pre,
                                                                            const StepConst c,
                                                                            unsigned *__restrict__ flag) {
    constexpr int AHEAD = zt_img_ahead(K);
    static_assert(AHEAD <= (K - 1) / 2, "image fetches must stay inside the volume");
    constexpr int NG = K / ZT_G;  // barrier groups in the ring
    static_assert(K % AHEAD == 0, "the image ring depth must divide the tap count");
    static_assert(K % ZT_G == 0, "the barrier group must divide the tap count");
    extern __shared__ __align__(128) unsigned char zsm[];
    float(*slot)[2][ZT_Y][2 * ZT_X] = reinterpret_cast<float(*)[2][ZT_Y][2 * ZT_X]>(zsm);
    uint64_t *full = reinterpret_cast<uint64_t *>(zsm + (size_t)K * ZT_SLOT_BYTES);
    uint64_t *empty = full + NG;
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
        for (int q = 0; q < NG; ++q) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], ZT_CONSUMERS);
        }
        fence_barrier_init();
    }
    __syncthreads();
    if (warp == ZT_CONSUMERS) {
        // producer: group g = planes g ZT_G .. g ZT_G + ZT_G - 1 (fewer at the
        // end) into slots (g mod NG) ZT_G + j once the consumers have released
        // the group NG before it
        if (lane == 0) {
            tensormap_acquire(map);
            const int ngroups = (L + ZT_G - 1) / ZT_G;
            for (int g = 0; g < ngroups; ++g) {
                const int q = g % NG;
                if (g >= NG && !mbar_wait(&empty[q], (unsigned)((g / NG) - 1) & 1u)) {
                    atomicOr(flag, kFlagTimeout);
                    break;
                }
                const int first = g * ZT_G, n = min(ZT_G, L - first);
                mbar_arrive_expect_tx(&full[q], (unsigned)n * ZT_SLOT_BYTES);
                for (int j = 0; j < n; ++j)
                    tma_load_4d(&slot[q * ZT_G + j][0][0][0], map, 2 * x0, y0, first + j, 0, &full[q]);
            }
        }
        return;
    }
    // consumer: column x, pair p (lanes 0-15 pair 0, 16-31 pair 1)
    const int yy = warp >> 1, xx = (warp & 1) * 16 + (lane & 15), p = lane >> 4;
    const int x = x0 + xx, y = y0 + yy;
    const bool act = x < Wv && y < Hv;
    const int r = c.r;
    const bool f32 = c.img_f32 != 0;
    const size_t esz = f32 ? 4 : 1;
    const size_t pl_bytes = (size_t)s.W * s.H * esz;  // image plane stride in bytes
    // this column's image address at output plane 0 (image plane r)
    const uintptr_t im0 = reinterpret_cast<uintptr_t>(s.img) +
                          (((size_t)r * s.H + (size_t)(y + r)) * s.W + (size_t)(x + r)) * esz;
    // The image word of output o: the float's bits, or the aligned 32-bit
    // word holding the byte (it lies in the byte's own 4-byte block, so it
    // never reaches another allocation).  Nothing reads the loaded register
    // until the value is needed AHEAD outputs later.  The fetches run at most
    // AHEAD <= r outputs past the last one, i.e. up to image plane
    // Lv - 1 + AHEAD + r < L: always inside the volume.
    auto image_word = [&](int o) -> unsigned {
        return act ? __ldg(reinterpret_cast<const unsigned *>((im0 + (size_t)o * pl_bytes) & ~(uintptr_t)3)) : 0u;
    };
    float *dbp = s.db + (size_t)y * s.Wp + x;
    const size_t db_plane = (size_t)s.Wp * Hv;
    const float2 *vsrc = reinterpret_cast<const float2 *>(&slot[0][p][yy][2 * xx]);
    constexpr int kSlot = (int)(ZT_SLOT_BYTES / sizeof(float2));
    unsigned img[AHEAD];
#pragma unroll
    for (int q = 0; q < AHEAD; ++q) img[q] = image_word(q);
    bool ok = true;
    float2 acc[K];
#pragma unroll
    for (int q = 0; q < K; ++q) acc[q] = make_float2(0.f, 0.f);
    // planes base .. base + K - 1: plane base + j sits in ring slot j, in
    // barrier group j / ZT_G with phase (base / K) & 1; z-output
    // o = base + j - (K - 1) uses accumulator (j + 1) mod K and image slot
    // (j + 1) mod AHEAD
    // `guard`: the last, partial block
    auto block = [&](int base, bool guard) {
        const unsigned ph = (unsigned)(base / K) & 1u;
#pragma unroll
        for (int j = 0; j < K; ++j) {
            const int i = base + j;
            if (guard && i >= L) break;
            if (j % ZT_G == 0 && ok && !mbar_wait(&full[j / ZT_G], ph)) {
                ok = false;
                atomicOr(flag, kFlagTimeout);
            }
            const float2 v = vsrc[j * kSlot];
            // the group is released after its last plane (or the volume's)
            if (j % ZT_G == ZT_G - 1 || i == L - 1) {
                __syncwarp();
                if (lane == 0) mbar_arrive(&empty[j / ZT_G]);
            }
#pragma unroll
            for (int tt = 0; tt < K; ++tt) {
                const int q = (j - tt + K) % K;
                if (tt == 0) acc[q] = fma2(v, c.taps2[0], make_float2(0.f, 0.f));
                else acc[q] = fma2(v, c.taps2[tt], acc[q]);
            }
            const int o = i - (K - 1);
            if (o >= 0) {
                const int m = (j + 1) % AHEAD;
                const unsigned w = img[m];
                const unsigned sh = 8u * (((unsigned)im0 + (unsigned)o * (unsigned)pl_bytes) & 3u);
                const float I = f32 ? __uint_as_float(w) : (float)((w >> sh) & 0xffu);
                img[m] = image_word(o + AHEAD);
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
