// rsf_internal.h -- data structures shared by the kernels and the C ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace rsf {

constexpr int MAXK = 128;  // largest supported tap count (sigma up to ~18)

// Kernel tilings (the launchers derive tile counts from them).
constexpr int XP_ROWS = 4;     // x-pass: warps per block
constexpr int XP_RPW = 8;      // x-pass: largest rows per warp (XP_ROWS apart; chosen per launch)
constexpr int YP_COLS = 128;   // y-pass: columns per block (one column of one pair per thread)
constexpr int YB_TX = 128;     // generic y-pass: columns per block
constexpr int YB_YB = 16;      // generic y-pass: outputs per thread along y
constexpr int ZP_PAIRS = 32;   // z-pass: column pairs per block (four lanes each)
constexpr int ZB_TX = 128;     // generic z-pass: columns per block
constexpr int ZB_ZB = 16;      // generic z-pass: outputs per thread along z
constexpr int ST_OX = 30;      // stencil: output columns per warp (lanes 1..30)
constexpr int ST_OY = 14;      // stencil: output rows per block (warps 1..14)
constexpr int ST_WARPS = ST_OY + 2;
constexpr int ST_ZC = 64;      // stencil: planes per block (chosen per launch: 32, 64 or ST_ZC_MAX)
constexpr int ST_ZC_MAX = 128;

// The x-pass lane width (outputs per lane) is chosen per launch from these.
constexpr int XB_CHOICES[2] = {5, 9};

// One sub-volume as the kernels see it.
//   xb: x-pass fields, each Wp x H x L   (row stride Wp)
//   yb: y-pass fields, each Wp x Hv x L
//   The specialised tap counts keep the fields as two float2 pair planes,
//   pair 0 (H, 1-H) and pair 1 (I H, I (1-H)); the run-time-k kernels as four
//   separate float planes (H, 1-H, I H, I (1-H)).
//   db: data factor lambda (e_out - e_in) of the valid region, Wp x Hv x Lv;
//       it reuses the x-pass storage, which is dead once the y-pass has run.
//       With the box e-term or the expanded data term it holds f_out and
//       f_in of the valid region (Wp x Hv x Lv each) followed by the data
//       factor of every voxel (W x H x L).
struct SubVolDev {
    float *phi[2];       // ping-pong level-set buffers
    const void *img;     // image, uint8 or float32
    float *xb;
    float *yb;
    float *db;
    int W, H, L;
    int Wv, Hv, Lv;      // valid extents of the blur (0: all border)
    int Wp;              // padded row stride of xb / yb / db (multiple of 4)
    int pad;
};

// Per-launch constants, passed by value (they live in the constant bank).
struct StepConst {
    float taps[MAXK];
    float2 taps2[MAXK];  // (g, g) pairs for the packed multiply-adds
    int k, r;
    float eps, dt, mu, nu, l1, l2;
    int lam_equal;
    int boundary;   // 0 reference (x = 0 wraps to the previous row), 1 clamp
    int img_f32;    // 1: image is float32, 0: uint8
    int nsv;        // number of sub-volumes in the table
    int xb_w;       // x-pass outputs per lane for this launch
    int xrpw;       // x-pass rows per warp for this launch
    int pairs;      // 1: x/y fields in float2 pair planes (specialised tap counts)
    int zc;         // stencil planes per block for this launch
    int box;        // e-term box radius (int)sigma2; 0: e = (I - f)^2
    int gauss;      // 1: expanded Gaussian data term (rsf_gauss.cu)
    int full_data;  // box or gauss: the z-pass stores the fits, the data factor of every voxel follows them
    float s3;       // gauss: the valid correlation of ones, K*1
    ptrdiff_t gdelta;  // gauss: offset (floats) of the scratch G from xb
    const void *ymaps;  // per sub-volume TMA map of the y-pass pair planes (TMAP_BYTES each), or null
};

// TMA tensor maps (CUtensorMap) as the kernels see them: 128 bytes each, in
// device memory aligned to 128 bytes.
constexpr int TMAP_BYTES = 128;
// Encodes the z-pass map of d's pair planes into `out` (host memory); false
// when the driver's encoder is unavailable or refuses the layout.
bool encode_pair_map(void *out, const SubVolDev &d);
bool tensor_maps_available();
bool tma_z_requested();

// Optional per-voxel debug outputs (8 fields, full-volume layout).
struct DebugOut {
    float *f;
    int64_t n;
};

constexpr int NKERN = 4;  // x-pass, y-pass, z-pass, stencil (timed separately)
// Block prefix arrays per batch: the NKERN kernels, then the expanded
// data term's gauss_x, second y-pass, gauss_z and gauss_border.
constexpr int NPRE = NKERN + 4;
constexpr int GX_T = 128;  // gauss_x: threads per block
constexpr int GX_NB = 4;   // gauss_x: x-outputs per thread
constexpr int GB_T = 256;  // gauss_border: voxels per block

// Bits of the per-workspace error flag the kernels set.
constexpr unsigned kFlagNonFinite = 1u;  // a non-finite value was written to phi
constexpr unsigned kFlagTimeout = 2u;    // a barrier wait gave up (a TMA copy did not complete)
constexpr unsigned kFlagAdjointNonFinite = 4u;  // rsf_step_adjoint produced a non-finite dL/dphi

// Tap counts with streaming (compile-time K) kernels.  Other tap counts, the
// debug step, the reference arithmetic and the box e-term use the
// run-time-k kernels.
inline bool is_specialised(int k) { return k == 21 || k == 29 || k == 35; }
inline int kernel_k(int k, int arith, bool debug, int box = 0, int gauss = 0) {
    return (is_specialised(k) && arith == 0 && !debug && box == 0 && gauss == 0) ? k : 0;
}
// Specialised tap counts whose z-pass can run fed by TMA (its image prefetch
// ring depth divides k).
inline bool tma_z(int kspec) { return kspec == 21 || kspec == 35; }
constexpr int MAX_BOX = 8;  // largest e-term box radius

// Per-launch tile shapes of a batch.
struct LaunchShape {
    int xb_w;   // x-pass outputs per lane
    int xrpw;   // x-pass rows per warp (1, 2, 4 or XP_RPW)
    int pairs;  // 1: x/y fields in float2 pair planes (specialised tap counts)
    int zt;     // 1: the z-pass loads planes with TMA (needs a map per sub-volume)
    int zc;     // stencil planes per block
    int gauss;  // 1: the expanded data term's kernels run (tiles NKERN .. NPRE - 1)
};
// whl: W, H, L of each sub-volume; kspec: kernel_k().
LaunchShape choose_shape(const int *whl, int n, int k, int kspec, int gauss = 0);
// Blocks each kernel needs for one sub-volume (kspec: kernel_k()).
void tile_counts(const SubVolDev &d, int kspec, const LaunchShape &sh, int tiles[NPRE]);
int choose_xb(const int *Wv, int n);
// Rows per warp of the x-pass: the most (up to XP_RPW) that still give
// every SM several blocks.
int choose_xrpw(const int *whl, int n, int k, int xb_w);
int choose_zc(const int *whl, int n);  // whl: W, H, L of each sub-volume
void valid_extents(int W, int H, int L, int k, int &Wv, int &Hv, int &Lv, int &Wp);

// One iteration.  With `ev` (NKERN + 1 events) the events are recorded before
// the first and after every kernel, for per-kernel device times.
cudaError_t launch_step(const SubVolDev *d_svs, const int *d_pre, const int *h_tot, const StepConst &c,
                        int parity, int arith, unsigned *d_flag, const DebugOut *dbg, cudaStream_t st,
                        cudaEvent_t *ev = nullptr);

cudaError_t configure_device();

// Streaming multiprocessors of the current device (cached per device; 152 on
// GB300), for grid caps and wave counts.
int sm_count();

// Sets the message rsf_last_error() returns on the calling thread.
void set_last_error(const char *msg);

// Per-kernel launchers; each tap specialisation lives in its own object file.
// One volume of an adjoint batch (rsf_adjoint.cu), N = W H L.
struct AdjVol {
    const float *phi;  // the step's input level set
    const void *img;
    const float *u;    // dL/dphi' of the step's output
    float *out;        // dL/dphi
    float *phi2;       // scratch, N floats
    float *xs, *ys;    // scratch, 4 N floats each
    int W, H, L;
    int Wv, Hv, Lv;    // valid blur extents; all > 0 or all 0
};
// Adjoint kernels with a block prefix array each (rsf_adjoint.cu): H, the
// recompute blurs x, y, z, the transposed blurs z, y, x, normals, pointwise
// terms, w, gather.
constexpr int NADJ = 11;
enum AdjKernel { ADJ_H, ADJ_BX, ADJ_BY, ADJ_BZ, ADJ_TZ, ADJ_TY, ADJ_TX, ADJ_NRM, ADJ_PT, ADJ_W, ADJ_G };
// Blocks of each adjoint kernel for one volume; with `streamed` the
// recompute (ADJ_H .. ADJ_BZ) runs in the forward step's kernels instead.
void adjoint_tiles(const AdjVol &v, bool streamed, int tiles[NADJ]);

#define RSF_DECLARE_K(K)                                                                                      \
    cudaError_t launch_xpass_##K(const SubVolDev *, const int *, int, const StepConst &, int, int, cudaStream_t); \
    cudaError_t config_xpass_##K();                                                                             \
    cudaError_t launch_ypass_##K(const SubVolDev *, const int *, int, const StepConst &, cudaStream_t);          \
    cudaError_t launch_zpass_##K(const SubVolDev *, const int *, int, const StepConst &, const DebugOut *,      \
                                 cudaStream_t);
RSF_DECLARE_K(0)
RSF_DECLARE_K(21)
RSF_DECLARE_K(29)
RSF_DECLARE_K(35)
#undef RSF_DECLARE_K
// The streaming z-pass with the adjoint's emit (pair planes, specialised k):
// sub-volume i of the table is volume i of `vols`.
cudaError_t launch_zpass_adjoint_21(const SubVolDev *, const int *, int, const StepConst &, const AdjVol *vols,
                                    cudaStream_t);
cudaError_t launch_zpass_adjoint_29(const SubVolDev *, const int *, int, const StepConst &, const AdjVol *vols,
                                    cudaStream_t);
cudaError_t launch_zpass_adjoint_35(const SubVolDev *, const int *, int, const StepConst &, const AdjVol *vols,
                                    cudaStream_t);
cudaError_t config_ztpass_21();
cudaError_t config_ztpass_35();
cudaError_t launch_ztpass_21(const SubVolDev *, const int *, int, const StepConst &, unsigned *flag, cudaStream_t);
cudaError_t launch_ztpass_35(const SubVolDev *, const int *, int, const StepConst &, unsigned *flag, cudaStream_t);
cudaError_t launch_stencil(const SubVolDev *, const int *, int, const StepConst &, int parity, int arith,
                           unsigned *flag, const DebugOut *dbg, cudaStream_t);
// Expanded data term (c.gauss): its four kernels after the z-pass; pre holds
// NPRE prefix arrays of n1 entries, tot their totals.
cudaError_t launch_gauss(const SubVolDev *, const int *pre, int n1, const int *tot, const StepConst &,
                         const DebugOut *dbg, cudaStream_t);
// Box e-term (c.box >= 1): data factor of every voxel, stencil tiling.
cudaError_t launch_box(const SubVolDev *, const int *, int, const StepConst &, const DebugOut *dbg, cudaStream_t);
// Reverse-mode derivative of one step for a batch of volumes (rsf_adjoint.cu).
// vols: n entries (device); pre: NADJ block prefix arrays of n + 1 entries
// (device); tot: their totals.  Parameter sums over the batch are added to
// grads[0..3] when grads is not null.
struct AdjScalars {
    float eps, dt, mu, nu, l1, l2;
    int boundary, img_f32;
};
cudaError_t launch_step_adjoint(const float *taps, int k, const AdjScalars &s, const AdjVol *vols, const int *pre,
                                int n, const int *tot, double *grads, unsigned *flag, cudaStream_t st);
// Reassembly (rsf_reassemble.cu): one evolved sub-volume placed in the output.
constexpr int RA_MAXCELLS = 64;  // grid cells per axis
struct TileDev {
    const float *phi;
    int x0, y0, z0;
    int W, H, L;
};
cudaError_t launch_reassemble(const TileDev *d_tiles, const int n[3], const int *const cb[3], const int *const lo[3],
                              const int *const hi[3], int mode, float *out, int W, int H, int L, cudaStream_t st);
// SM copy between device-accessible addresses (rsf_copy.cu).
cudaError_t launch_copy(void *dst, const void *src, size_t bytes, cudaStream_t st);
// Signed distance of {seed > thr}; scratch holds 3 * W*H*L words.
cudaError_t launch_signed_distance(const void *seed, int f32, float thr, float *phi, int W, int H, int L,
                                   unsigned *scratch, cudaStream_t st);

}  // namespace rsf
