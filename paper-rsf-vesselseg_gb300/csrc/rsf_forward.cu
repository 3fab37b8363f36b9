// rsf_forward.cu -- one RSF iteration on the device, three kernels per step.
//
//   x-pass  : phi, I -> H, 1-H, I*H, I*(1-H) (pointwise, kernel.cu:210-298)
//             and their valid correlation along x (kernel.cu:1000-1014)
//   y-pass  : valid correlation along y (kernel.cu:1017-1031)
//   update  : valid correlation along z (kernel.cu:1035-1049), border band
//             := 30/30 (kernel.cu:300-325), f = blur(I H)/blur(H)
//             (kernel.cu:191-207), e = (I - f)^2 (kernel.cu:25-55),
//             gradient / |gradient| / normalised gradient / curvature /
//             "Laplacian" (kernel.cu:57-125, 173-189, 630-933), delta
//             (kernel.cu:265-280) and the explicit update (kernel.cu:365-387),
//             fused into one z-streaming kernel that writes phi once.
//
// Every kernel takes the whole batch: a table of sub-volumes and, per kernel,
// a prefix sum of the blocks each sub-volume needs.  Block b finds its
// sub-volume by binary search.  A single volume is a batch of one.
//
// Summation order is the reference's: each blurred value is accumulated with
// fused multiply-adds from 0 over ascending taps, x first, then y, then z.
#include <cuda_runtime.h>
#include <stdint.h>

#include "rsf_arith.cuh"
#include "rsf_internal.h"

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

// ---------------------------------------------------------------------------
// x-pass.  One warp per image row; a lane produces XP_XB consecutive outputs
// of each field from a shared-memory copy of the row (stride XP_XB is odd, so
// the lanes' reads fall in distinct banks), results staged in shared memory
// and written coalesced.
// ---------------------------------------------------------------------------
template <int K, Arith A>
__global__ void __launch_bounds__(XP_ROWS * 32) xpass_kernel(const SubVolDev *__restrict__ svs,
                                                              const int *__restrict__ pre,
                                                              const StepConst c, int parity) {
    extern __shared__ float sm[];
    const int k = K > 0 ? K : c.k;
    const int span = XP_TX + k - 1;
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int ntx = (s.Wv + XP_TX - 1) / XP_TX, nty = (s.H + XP_ROWS - 1) / XP_ROWS;
    const int tx = t % ntx;
    t /= ntx;
    const int ty = t % nty;
    const int z = t / nty;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y = ty * XP_ROWS + warp;
    float *taps = sm + XP_ROWS * (4 * span + 4 * XP_TX);
    if (K == 0) {
        for (int i = threadIdx.x; i < k; i += blockDim.x) taps[i] = c.taps[i];
        __syncthreads();
    }
    if (y >= s.H) return;
    float *in = sm + warp * (4 * span + 4 * XP_TX);
    float *out = in + 4 * span;
    const int x0 = tx * XP_TX;
    const size_t row = ((size_t)z * s.H + y) * s.W;
    const float *phi = (parity ? s.phi[1] : s.phi[0]) + row;
    for (int e = lane; e < span; e += 32) {
        const int x = x0 + e;
        float h = 0.0f, I = 0.0f;
        if (x < s.W) {
            h = heaviside<A>(__ldg(phi + x), c.eps);
            I = load_img(s.img, row + x, c.img_f32);
        }
        const float hi = __fsub_rn(1.0f, h);
        in[F_H * span + e] = h;
        in[F_HI * span + e] = hi;
        in[F_IH * span + e] = __fmul_rn(I, h);
        in[F_IHI * span + e] = __fmul_rn(I, hi);
    }
    __syncwarp();
#pragma unroll 1
    for (int f = 0; f < 4; ++f) {
        const float *src = in + f * span + XP_XB * lane;
        float acc[XP_XB];
#pragma unroll
        for (int m = 0; m < XP_XB; ++m) acc[m] = 0.0f;
        if constexpr (K > 0) {
#pragma unroll
            for (int q = 0; q < XP_XB + K - 1; ++q) {
                const float v = src[q];
#pragma unroll
                for (int m = 0; m < XP_XB; ++m) {
                    const int tt = q - m;
                    if (tt >= 0 && tt < K) acc[m] = __fmaf_rn(v, c.taps[tt], acc[m]);
                }
            }
        } else {
            for (int q = 0; q < XP_XB + k - 1; ++q) {
                const float v = src[q];
#pragma unroll
                for (int m = 0; m < XP_XB; ++m) {
                    const int tt = q - m;
                    if (tt >= 0 && tt < k) acc[m] = __fmaf_rn(v, taps[tt], acc[m]);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < XP_XB; ++m) out[f * XP_TX + XP_XB * lane + m] = acc[m];
    }
    __syncwarp();
    const size_t fstride = (size_t)s.Wv * s.H * s.L;
    const size_t orow = ((size_t)z * s.H + y) * s.Wv;
#pragma unroll 1
    for (int f = 0; f < 4; ++f)
        for (int e = lane; e < XP_TX; e += 32) {
            const int x = x0 + e;
            if (x < s.Wv) s.xb[f * fstride + orow + x] = out[f * XP_TX + e];
        }
}

// ---------------------------------------------------------------------------
// Register-blocked valid correlation of NB consecutive outputs along a
// strided axis: out[m] = sum_t in[(start + m + t) * stride] g[t], taps
// ascending, inputs outside [0, n) read as 0 (they only feed outputs the
// caller discards).
// ---------------------------------------------------------------------------
template <int K, int NB>
__device__ __forceinline__ void conv_block(const float *__restrict__ base, size_t stride, int start,
                                           int n, const StepConst &c, const float *taps_s, int k,
                                           float (&acc)[NB]) {
#pragma unroll
    for (int m = 0; m < NB; ++m) acc[m] = 0.0f;
    if constexpr (K > 0) {
#pragma unroll
        for (int q = 0; q < NB + K - 1; ++q) {
            const int p = start + q;
            const float v = (p >= 0 && p < n) ? __ldg(base + (size_t)p * stride) : 0.0f;
#pragma unroll
            for (int m = 0; m < NB; ++m) {
                const int tt = q - m;
                if (tt >= 0 && tt < K) acc[m] = __fmaf_rn(v, c.taps[tt], acc[m]);
            }
        }
    } else {
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
}

// ---------------------------------------------------------------------------
// y-pass.  One thread per x column of a YP_YB-row chunk; loads are coalesced
// across the block.
// ---------------------------------------------------------------------------
template <int K>
__global__ void __launch_bounds__(YP_TX) ypass_kernel(const SubVolDev *__restrict__ svs,
                                                      const int *__restrict__ pre, const StepConst c) {
    __shared__ float taps_s[K == 0 ? MAXK : 1];
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int ntx = (s.Wv + YP_TX - 1) / YP_TX, nty = (s.Hv + YP_YB - 1) / YP_YB;
    const int tx = t % ntx;
    t /= ntx;
    const int ty = t % nty;
    const int z = t / nty;
    const int k = K > 0 ? K : c.k;
    if (K == 0) {
        for (int i = threadIdx.x; i < k; i += blockDim.x) taps_s[i] = c.taps[i];
        __syncthreads();
    }
    const int x = tx * YP_TX + threadIdx.x;
    if (x >= s.Wv) return;
    const int y0 = ty * YP_YB;
    const size_t fin = (size_t)s.Wv * s.H * s.L, fout = (size_t)s.Wv * s.Hv * s.L;
#pragma unroll 1
    for (int f = 0; f < 4; ++f) {
        const float *src = s.xb + f * fin + (size_t)z * s.H * s.Wv + x;
        float acc[YP_YB];
        conv_block<K, YP_YB>(src, (size_t)s.Wv, y0, s.H, c, taps_s, k, acc);
        float *dst = s.yb + f * fout + ((size_t)z * s.Hv) * s.Wv + x;
#pragma unroll
        for (int m = 0; m < YP_YB; ++m)
            if (y0 + m < s.Hv) dst[(size_t)(y0 + m) * s.Wv] = acc[m];
    }
}

// ---------------------------------------------------------------------------
// Update kernel: a UP_TX x UP_TY tile of columns, UP_ZB planes deep.
//  phase 1: per column, the z correlation of the four y-pass fields for the
//           block's planes (register blocked), the local fits and the data
//           factor lambda (e_out - e_in), kept in shared memory;
//  phase 2: streams z through a ring of phi planes (2-voxel halo) and a ring
//           of gradient / normalised-gradient planes (1-voxel halo), forms
//           curvature and "Laplacian" with the reference's boundary rules and
//           writes the updated phi.
// ---------------------------------------------------------------------------
struct GN {
    float gx, gy, gz, nx, ny, nz;
};

// Gradient and normalised gradient at (x, y, z) read straight from global
// memory with the boundary rules of kernel.cu:57-125 (used for the previous-
// row neighbour of x = 0 in the reference boundary mode).
template <Arith A>
__device__ __forceinline__ GN gn_global(const float *__restrict__ phi, int x, int y, int z, int W, int H,
                                        int L, int boundary) {
    const size_t WH = (size_t)W * H;
    auto at = [&](int xx, int yy, int zz) { return __ldg(phi + (size_t)zz * WH + (size_t)yy * W + xx); };
    const float c0 = at(x, y, z);
    float xl, xr;
    if (x > 0) xl = at(x - 1, y, z);
    else if (boundary == 0) {
        if (y > 0) xl = at(W - 1, y - 1, z);
        else if (z > 0) xl = at(W - 1, H - 1, z - 1);
        else xl = c0;
    } else xl = c0;
    xr = x < W - 1 ? at(x + 1, y, z) : c0;
    const float yl = y > 0 ? at(x, y - 1, z) : c0, yr = y < H - 1 ? at(x, y + 1, z) : c0;
    const float zl = z > 0 ? at(x, y, z - 1) : c0, zr = z < L - 1 ? at(x, y, z + 1) : c0;
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

template <int K, Arith A, bool DEBUG>
__global__ void __launch_bounds__(UP_TX *UP_TY) update_kernel(const SubVolDev *__restrict__ svs,
                                                             const int *__restrict__ pre,
                                                             const StepConst c, int parity,
                                                             unsigned *__restrict__ flag, DebugOut dbg) {
    constexpr int PX = UP_TX + 4, PY = UP_TY + 4, GXN = UP_TX + 2, GYN = UP_TY + 2;
    constexpr int NT = UP_TX * UP_TY;
    __shared__ float phis[4][PY * PX];
    __shared__ float gns[3][6][GYN * GXN];
    __shared__ float dat[UP_ZB][NT];
    __shared__ float taps_s[K == 0 ? MAXK : 1];

    const int tid = threadIdx.x;
    const int lx = tid % UP_TX, ly = tid / UP_TX;
    const int b = blockIdx.x;
    const int sv = find_sv(pre, c.nsv, b);
    const SubVolDev s = svs[sv];
    int t = b - __ldg(pre + sv);
    const int W = s.W, H = s.H, L = s.L;
    const int ntx = (W + UP_TX - 1) / UP_TX, nty = (H + UP_TY - 1) / UP_TY;
    const int tx = t % ntx;
    t /= ntx;
    const int ty = t % nty;
    const int tz = t / nty;
    const int x0 = tx * UP_TX, y0 = ty * UP_TY, z0 = tz * UP_ZB;
    const int x = x0 + lx, y = y0 + ly;
    const bool active = x < W && y < H;
    const size_t WH = (size_t)W * H;
    const float *__restrict__ phi = parity ? s.phi[1] : s.phi[0];
    float *__restrict__ phi_out = parity ? s.phi[0] : s.phi[1];
    const int k = K > 0 ? K : c.k;
    const int r = c.r;
    const int zend = min(z0 + UP_ZB, L);
    if (K == 0)
        for (int i = tid; i < k; i += NT) taps_s[i] = c.taps[i];
    __syncthreads();

    // ---------------- phase 1: local fits and data factor ----------------
    {
        const bool inxy = active && s.Wv > 0 && s.Hv > 0 && s.Lv > 0 && x >= r && x < W - r && y >= r &&
                          y < H - r;
        float fo[UP_ZB], fi[UP_ZB];
#pragma unroll
        for (int m = 0; m < UP_ZB; ++m) fo[m] = fi[m] = 1.0f;
        if (inxy) {
            const size_t fstride = (size_t)s.Wv * s.Hv * L;
            const size_t pstride = (size_t)s.Wv * s.Hv;
            const float *col = s.yb + (size_t)(y - r) * s.Wv + (x - r);
            float num[UP_ZB], den[UP_ZB];
            conv_block<K, UP_ZB>(col + F_IH * fstride, pstride, z0 - r, L, c, taps_s, k, num);
            conv_block<K, UP_ZB>(col + F_H * fstride, pstride, z0 - r, L, c, taps_s, k, den);
#pragma unroll
            for (int m = 0; m < UP_ZB; ++m) {
                const int z = z0 + m;
                if (z >= r && z < L - r) fo[m] = __fdiv_rn(num[m], den[m]);
            }
            conv_block<K, UP_ZB>(col + F_IHI * fstride, pstride, z0 - r, L, c, taps_s, k, num);
            conv_block<K, UP_ZB>(col + F_HI * fstride, pstride, z0 - r, L, c, taps_s, k, den);
#pragma unroll
            for (int m = 0; m < UP_ZB; ++m) {
                const int z = z0 + m;
                if (z >= r && z < L - r) fi[m] = __fdiv_rn(num[m], den[m]);
            }
        }
        if (active) {
#pragma unroll
            for (int m = 0; m < UP_ZB; ++m) {
                const int z = z0 + m;
                if (z < L) {
                    const size_t vi = (size_t)z * WH + (size_t)y * W + x;
                    const float I = load_img(s.img, vi, c.img_f32);
                    const float d_o = __fsub_rn(I, fo[m]), d_i = __fsub_rn(I, fi[m]);
                    const float eo = __fmul_rn(d_o, d_o), ei = __fmul_rn(d_i, d_i);
                    dat[m][tid] = data_factor(eo, ei, c.l1, c.l2, c.lam_equal != 0);
                    if constexpr (DEBUG) {
                        dbg.f[0 * dbg.n + vi] = fo[m];
                        dbg.f[1 * dbg.n + vi] = fi[m];
                        dbg.f[2 * dbg.n + vi] = eo;
                        dbg.f[3 * dbg.n + vi] = ei;
                    }
                }
            }
        }
    }

    // ---------------- phase 2: stencils and update ----------------
    auto load_plane = [&](int zp) {
        float *dst = phis[zp & 3];
        const float *src = phi + (size_t)zp * WH;
        for (int e = tid; e < PX * PY; e += NT) {
            const int gx = x0 - 2 + e % PX, gy = y0 - 2 + e / PX;
            float v = 0.0f;
            if (gx >= 0 && gx < W && gy >= 0 && gy < H) v = __ldg(src + (size_t)gy * W + gx);
            dst[e] = v;
        }
    };
    // previous linear element of (0, yy, zz): reference rule for x = 0
    auto prev_phi = [&](int yy, int zz, float self) {
        if (yy > 0) return __ldg(phi + (size_t)zz * WH + (size_t)(yy - 1) * W + (W - 1));
        if (zz > 0) return __ldg(phi + (size_t)(zz - 1) * WH + (size_t)(H - 1) * W + (W - 1));
        return self;
    };

    const int zs = max(z0 - 1, 0), ze = min(z0 + UP_ZB, L - 1);
    if (zs > 0) load_plane(zs - 1);
    load_plane(zs);
    for (int zz = zs; zz <= ze; ++zz) {
        if (zz + 1 < L) load_plane(zz + 1);
        __syncthreads();
        // gradient and normalised gradient of plane zz over the tile + 1 halo
        {
            const float *P = phis[zz & 3];
            const float *Pz_l = phis[(zz > 0 ? zz - 1 : zz) & 3];
            const float *Pz_r = phis[(zz < L - 1 ? zz + 1 : zz) & 3];
            float *G = &gns[zz % 3][0][0];
            for (int e = tid; e < GXN * GYN; e += NT) {
                const int gxl = e % GXN, gyl = e / GXN;
                const int gx = x0 - 1 + gxl, gy = y0 - 1 + gyl;
                GN g = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                if (gx >= 0 && gx < W && gy >= 0 && gy < H) {
                    const int pc = (gyl + 1) * PX + (gxl + 1);
                    const float c0 = P[pc];
                    float xl;
                    if (gx > 0) xl = P[pc - 1];
                    else xl = (c.boundary == 0) ? prev_phi(gy, zz, c0) : c0;
                    const float xr = gx < W - 1 ? P[pc + 1] : c0;
                    const float yl = gy > 0 ? P[pc - PX] : c0, yr = gy < H - 1 ? P[pc + PX] : c0;
                    g.gx = half_diff(xr, xl);
                    g.gy = half_diff(yr, yl);
                    g.gz = half_diff(Pz_r[pc], Pz_l[pc]);
                    const NormDen d = norm_den<A>(grad_mag(g.gx, g.gy, g.gz));
                    g.nx = normalise<A>(g.gx, d);
                    g.ny = normalise<A>(g.gy, d);
                    g.nz = normalise<A>(g.gz, d);
                }
                G[0 * GXN * GYN + e] = g.gx;
                G[1 * GXN * GYN + e] = g.gy;
                G[2 * GXN * GYN + e] = g.gz;
                G[3 * GXN * GYN + e] = g.nx;
                G[4 * GXN * GYN + e] = g.ny;
                G[5 * GXN * GYN + e] = g.nz;
            }
        }
        __syncthreads();
        // outputs: plane zz-1, and plane L-1 once its last neighbour exists
        for (int pass = 0; pass < 2; ++pass) {
            const int zo = pass == 0 ? zz - 1 : zz;
            if (pass == 1 && zz != L - 1) break;
            if (zo < z0 || zo >= zend || !active) continue;
            constexpr int GP = GXN * GYN;
            const float *G0 = &gns[zo % 3][0][0];
            const float *Gl = &gns[(zo > 0 ? zo - 1 : zo) % 3][0][0];
            const float *Gr = &gns[(zo < L - 1 ? zo + 1 : zo) % 3][0][0];
            const int cc = (ly + 1) * GXN + (lx + 1);
            float nxl, gxl;
            if (x > 0) {
                nxl = G0[3 * GP + cc - 1];
                gxl = G0[0 * GP + cc - 1];
            } else if (c.boundary == 0 && (y > 0 || zo > 0)) {
                const GN w = y > 0 ? gn_global<A>(phi, W - 1, y - 1, zo, W, H, L, c.boundary)
                                   : gn_global<A>(phi, W - 1, H - 1, zo - 1, W, H, L, c.boundary);
                nxl = w.nx;
                gxl = w.gx;
            } else {
                nxl = G0[3 * GP + cc];
                gxl = G0[0 * GP + cc];
            }
            const int cxr = x < W - 1 ? cc + 1 : cc;
            const int cyl = y > 0 ? cc - GXN : cc, cyr = y < H - 1 ? cc + GXN : cc;
            const float dxn = half_diff(G0[3 * GP + cxr], nxl);
            const float dyn = half_diff(G0[4 * GP + cyr], G0[4 * GP + cyl]);
            const float dzn = half_diff(Gr[5 * GP + cc], Gl[5 * GP + cc]);
            const float dxg = half_diff(G0[0 * GP + cxr], gxl);
            const float dyg = half_diff(G0[1 * GP + cyr], G0[1 * GP + cyl]);
            const float dzg = half_diff(Gr[2 * GP + cc], Gl[2 * GP + cc]);
            const float kap = __fadd_rn(__fadd_rn(dxn, dyn), dzn);
            const float lap = __fadd_rn(__fadd_rn(dxg, dyg), dzg);
            const float pc = phis[zo & 3][(ly + 2) * PX + (lx + 2)];
            const float dh = dirac<A>(pc, c.eps);
            const float out = update_phi(pc, dh, dat[zo - z0][tid], kap, lap, c.dt, c.nu, c.mu);
            const size_t vi = (size_t)zo * WH + (size_t)y * W + x;
            phi_out[vi] = out;
            if (!isfinite(out)) atomicOr(flag, 1u);
            if constexpr (DEBUG) {
                dbg.f[4 * dbg.n + vi] = dh;
                dbg.f[5 * dbg.n + vi] = kap;
                dbg.f[6 * dbg.n + vi] = lap;
                dbg.f[7 * dbg.n + vi] = grad_mag(G0[0 * GP + cc], G0[1 * GP + cc], G0[2 * GP + cc]);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
void tile_counts(int W, int H, int L, int k, int tiles[3], int &Wv, int &Hv, int &Lv) {
    Wv = W - k + 1;
    Hv = H - k + 1;
    Lv = L - k + 1;
    const bool valid = Wv > 0 && Hv > 0 && Lv > 0;
    if (!valid) Wv = Hv = Lv = 0;
    tiles[0] = valid ? ((Wv + XP_TX - 1) / XP_TX) * ((H + XP_ROWS - 1) / XP_ROWS) * L : 0;
    tiles[1] = valid ? ((Wv + YP_TX - 1) / YP_TX) * ((Hv + YP_YB - 1) / YP_YB) * L : 0;
    tiles[2] = ((W + UP_TX - 1) / UP_TX) * ((H + UP_TY - 1) / UP_TY) * ((L + UP_ZB - 1) / UP_ZB);
}

static size_t xpass_smem(int k, bool runtime_k) {
    const int span = XP_TX + k - 1;
    return sizeof(float) * ((size_t)XP_ROWS * (4 * span + 4 * XP_TX) + (runtime_k ? MAXK : 0));
}

template <int K, Arith A>
static cudaError_t run_xpass(const SubVolDev *svs, const int *pre, int blocks, const StepConst &c, int parity,
                             cudaStream_t st) {
    const size_t smem = xpass_smem(K > 0 ? K : c.k, K == 0);
    xpass_kernel<K, A><<<blocks, XP_ROWS * 32, smem, st>>>(svs, pre, c, parity);
    return cudaGetLastError();
}

template <int K, Arith A>
static cudaError_t allow_xpass_smem() {
    return cudaFuncSetAttribute(xpass_kernel<K, A>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)xpass_smem(MAXK, true));
}

// Raises the dynamic shared-memory limit of every x-pass instantiation on the
// current device; called once per workspace, outside any stream capture.
cudaError_t configure_device() {
    cudaError_t e = allow_xpass_smem<0, Arith::Portable>();
    if (e == cudaSuccess) e = allow_xpass_smem<0, Arith::Reference>();
    if (e == cudaSuccess) e = allow_xpass_smem<21, Arith::Portable>();
    if (e == cudaSuccess) e = allow_xpass_smem<29, Arith::Portable>();
    if (e == cudaSuccess) e = allow_xpass_smem<35, Arith::Portable>();
    return e;
}

template <int K, Arith A, bool DBG>
static cudaError_t run_pipeline(const SubVolDev *svs, const int *pre, const int *tot, const StepConst &c,
                                int parity, unsigned *flag, const DebugOut &dbg, cudaStream_t st) {
    const int nsv1 = c.nsv + 1;
    cudaError_t e = cudaSuccess;
    if (tot[0] > 0) {
        e = run_xpass<K, A>(svs, pre, tot[0], c, parity, st);
        if (e != cudaSuccess) return e;
    }
    if (tot[1] > 0) {
        ypass_kernel<K><<<tot[1], YP_TX, 0, st>>>(svs, pre + nsv1, c);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (tot[2] > 0) {
        update_kernel<K, A, DBG><<<tot[2], UP_TX * UP_TY, 0, st>>>(svs, pre + 2 * nsv1, c, parity, flag, dbg);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t launch_step(const SubVolDev *d_svs, const int *d_pre, const int *h_pre_tot, const StepConst &c,
                        int parity, int arith, unsigned *d_flag, const DebugOut *dbg, cudaStream_t st) {
    const DebugOut none = {nullptr, 0};
    if (dbg != nullptr) {
        if (arith == 1) return run_pipeline<0, Arith::Reference, true>(d_svs, d_pre, h_pre_tot, c, parity, d_flag, *dbg, st);
        return run_pipeline<0, Arith::Portable, true>(d_svs, d_pre, h_pre_tot, c, parity, d_flag, *dbg, st);
    }
    if (arith == 1) return run_pipeline<0, Arith::Reference, false>(d_svs, d_pre, h_pre_tot, c, parity, d_flag, none, st);
    switch (c.k) {
        case 21: return run_pipeline<21, Arith::Portable, false>(d_svs, d_pre, h_pre_tot, c, parity, d_flag, none, st);
        case 29: return run_pipeline<29, Arith::Portable, false>(d_svs, d_pre, h_pre_tot, c, parity, d_flag, none, st);
        case 35: return run_pipeline<35, Arith::Portable, false>(d_svs, d_pre, h_pre_tot, c, parity, d_flag, none, st);
        default: return run_pipeline<0, Arith::Portable, false>(d_svs, d_pre, h_pre_tot, c, parity, d_flag, none, st);
    }
}

}  // namespace rsf
