// rsf_internal.h -- data structures shared by the kernels and the C ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rsf {

constexpr int MAXK = 128;  // largest supported tap count (sigma up to ~18)

// Tilings (fixed at compile time; the launchers derive tile counts from them).
constexpr int XP_ROWS = 8;    // x-pass: rows per block (one warp per row)
constexpr int XP_XB = 5;      // x-pass: outputs per lane (odd: conflict-free smem)
constexpr int XP_TX = 32 * XP_XB;
constexpr int YP_TX = 128;    // y-pass: threads along x
constexpr int YP_YB = 16;     // y-pass: outputs per thread along y
constexpr int UP_TX = 32;     // update: tile width (x)
constexpr int UP_TY = 8;      // update: tile height (y)
constexpr int UP_ZB = 16;     // update: planes per block (z)

// One sub-volume as the kernels see it.
struct SubVolDev {
    float *phi[2];       // ping-pong level-set buffers
    const void *img;     // image, uint8 or float32
    float *xb;           // 4 fields of the x-pass, each Wv*H*L
    float *yb;           // 4 fields of the y-pass, each Wv*Hv*L
    int W, H, L;
    int Wv, Hv, Lv;      // valid extents of the blur (<= 0: all border)
    int tiles[3];        // blocks of x-pass, y-pass, update
    int pad;
};

// Per-launch constants, passed by value (they live in the constant bank).
struct StepConst {
    float taps[MAXK];
    int k, r;
    float eps, dt, mu, nu, l1, l2;
    int lam_equal;
    int boundary;   // 0 reference (x = 0 wraps to the previous row), 1 clamp
    int img_f32;    // 1: image is float32, 0: uint8
    int nsv;        // number of sub-volumes in the table
};

// Optional per-voxel debug outputs of the update kernel (8 fields).
struct DebugOut {
    float *f;       // 8 * N floats, field-major
    int64_t n;
};

cudaError_t launch_step(const SubVolDev *d_svs, const int *d_pre, const int *h_pre_tot,
                        const StepConst &c, int parity, int arith, unsigned *d_flag,
                        const DebugOut *dbg, cudaStream_t st);

cudaError_t configure_device();

void tile_counts(int W, int H, int L, int k, int tiles[3], int &Wv, int &Hv, int &Lv);

}  // namespace rsf
