// rsf_reassemble.cu -- stitches evolved sub-volumes back into one volume.
//
// The reference's pipeline stitches with scripts that do not ship
// (reassemble.py, README.md:9); the one present, interpolating_volumes.py:10-40,
// blends two volumes that overlap along one axis with weights (1 - a, a),
// a = 0 .. 1 in equal steps across the overlap.  Here the sub-volumes form a
// grid (core boxes that partition the volume, each grown by a halo and
// clipped at the faces) and every output voxel is gathered on the device:
//   core  (mode 0): the value of the sub-volume whose core holds the voxel;
//   blend (mode 1): per axis, a sub-volume's weight rises linearly across its
//                   overlap with the previous one and falls across its overlap
//                   with the next, with the same steps as the reference's
//                   blend; the weight of a sub-volume is the product over the
//                   axes and the output is sum(w phi) / sum(w).  Two volumes
//                   overlapping along one axis give the reference's blend.
// One thread per output voxel, x fastest, so reads of each sub-volume row and
// the output writes are coalesced; the grid geometry rides in the kernel
// parameters and the sub-volume table in device memory.
#include <cuda_runtime.h>

#include "rsf_internal.h"

namespace rsf {
namespace {

constexpr int kThreads = 256;

struct ReasmConst {
    int n[3];                        // cells per axis (x, y, z)
    int ext[3];                      // output extents (W, H, L)
    int mode;
    int cb[3][RA_MAXCELLS + 1];      // core boundaries per axis
    int lo[3][RA_MAXCELLS];          // sub-volume extent per axis and cell
    int hi[3][RA_MAXCELLS];
};

__device__ __forceinline__ int cell_of(const ReasmConst &c, int a, int p) {
    int lo = 0, hi = c.n[a] - 1;  // largest cell whose lower core bound is <= p
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (c.cb[a][mid] <= p) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ float tile_at(const TileDev &t, int x, int y, int z) {
    return t.phi[((long long)(z - t.z0) * t.H + (y - t.y0)) * t.W + (x - t.x0)];
}

// Blend weight of cell `ci` along axis a at coordinate p (0 if p is outside).
__device__ __forceinline__ float axis_weight(const ReasmConst &c, int a, int ci, int p) {
    const int lo = c.lo[a][ci], hi = c.hi[a][ci];
    if (p < lo || p >= hi) return 0.0f;
    float w = 1.0f;
    if (ci > 0 && c.hi[a][ci - 1] > lo && p < c.hi[a][ci - 1]) {
        const int ov = c.hi[a][ci - 1] - lo;
        w *= ov > 1 ? (float)(p - lo) / (float)(ov - 1) : 0.0f;
    }
    if (ci + 1 < c.n[a] && c.lo[a][ci + 1] < hi && p >= c.lo[a][ci + 1]) {
        const int ov = hi - c.lo[a][ci + 1];
        w *= ov > 1 ? (float)(hi - 1 - p) / (float)(ov - 1) : 1.0f;
    }
    return w;
}

__global__ void __launch_bounds__(kThreads) reassemble_kernel(ReasmConst c, const TileDev *tiles, float *out) {
    const long long N = (long long)c.ext[0] * c.ext[1] * c.ext[2];
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < N; i += (long long)gridDim.x * kThreads) {
        const int x = (int)(i % c.ext[0]);
        const long long r = i / c.ext[0];
        const int y = (int)(r % c.ext[1]);
        const int z = (int)(r / c.ext[1]);
        const int ix = cell_of(c, 0, x), iy = cell_of(c, 1, y), iz = cell_of(c, 2, z);
        if (c.mode == 0) {
            out[i] = tile_at(tiles[((long long)iz * c.n[1] + iy) * c.n[0] + ix], x, y, z);
            continue;
        }
        float acc = 0.0f, wsum = 0.0f;
        for (int dz = -1; dz <= 1; dz++) {
            const int cz = iz + dz;
            if (cz < 0 || cz >= c.n[2]) continue;
            const float wz = axis_weight(c, 2, cz, z);
            if (wz == 0.0f) continue;
            for (int dy = -1; dy <= 1; dy++) {
                const int cy = iy + dy;
                if (cy < 0 || cy >= c.n[1]) continue;
                const float wy = axis_weight(c, 1, cy, y);
                if (wy == 0.0f) continue;
                for (int dx = -1; dx <= 1; dx++) {
                    const int cx = ix + dx;
                    if (cx < 0 || cx >= c.n[0]) continue;
                    const float wx = axis_weight(c, 0, cx, x);
                    if (wx == 0.0f) continue;
                    const float w = wz * wy * wx;
                    acc = fmaf(w, tile_at(tiles[((long long)cz * c.n[1] + cy) * c.n[0] + cx], x, y, z), acc);
                    wsum += w;
                }
            }
        }
        out[i] = acc / wsum;
    }
}

}  // namespace

cudaError_t launch_reassemble(const TileDev *d_tiles, const int n[3], const int *const cb[3], const int *const lo[3],
                              const int *const hi[3], int mode, float *out, int W, int H, int L, cudaStream_t st) {
    ReasmConst c;
    c.ext[0] = W;
    c.ext[1] = H;
    c.ext[2] = L;
    c.mode = mode;
    for (int a = 0; a < 3; a++) {
        c.n[a] = n[a];
        for (int j = 0; j <= RA_MAXCELLS; j++) c.cb[a][j] = j <= n[a] ? cb[a][j] : 0;
        for (int j = 0; j < RA_MAXCELLS; j++) {
            c.lo[a][j] = j < n[a] ? lo[a][j] : 0;
            c.hi[a][j] = j < n[a] ? hi[a][j] : 0;
        }
    }
    const long long N = (long long)W * H * L;
    long long blocks = (N + kThreads - 1) / kThreads;
    if (blocks > 32LL * sm_count()) blocks = 32LL * sm_count();
    reassemble_kernel<<<(unsigned)blocks, kThreads, 0, st>>>(c, d_tiles, out);
    return cudaGetLastError();
}

}  // namespace rsf
