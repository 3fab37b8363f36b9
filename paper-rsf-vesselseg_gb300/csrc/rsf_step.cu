// rsf_step.cu -- host side of one RSF iteration: tilings and the launch
// sequence x-pass -> y-pass -> z-pass -> stencil.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "rsf_internal.h"
#include "rsf_zt.cuh"

namespace rsf {

int sm_count() {
    constexpr int kMaxDevices = 64;
    static std::atomic<int> cache[kMaxDevices];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return 1;
    }
    int n = cache[dev].load(std::memory_order_relaxed);
    if (n > 0) return n;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1) {
        cudaGetLastError();
        return 1;
    }
    cache[dev].store(n, std::memory_order_relaxed);
    return n;
}

void valid_extents(int W, int H, int L, int k, int &Wv, int &Hv, int &Lv, int &Wp) {
    Wv = W - k + 1;
    Hv = H - k + 1;
    Lv = L - k + 1;
    if (Wv <= 0 || Hv <= 0 || Lv <= 0) Wv = Hv = Lv = 0;
    Wp = (Wv + 3) & ~3;
}

// Lane width of the x-pass that computes the fewest wasted outputs.
int choose_xb(const int *Wv, int n) {
    int best = XB_CHOICES[0];
    long long best_cost = -1;
    for (int xb : XB_CHOICES) {
        const long long xt = 32LL * xb;
        long long cost = 0;
        for (int i = 0; i < n; i++) cost += ((Wv[i] + xt - 1) / xt) * xt;
        if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            best = xb;
        }
    }
    return best;
}

// Stencil planes per block: the most of ST_ZC_MAX, ST_ZC and ST_ZC / 2 that
// still gives four waves of blocks (two resident per SM); each block
// recomputes the gradient of two planes before its first output, so deeper
// blocks waste less (8.06 against 8.26 ms per launch on the 48-sub-volume
// batch for 128 against 64 planes).
int choose_zc(const int *whl, int n) {
    int zc = ST_ZC_MAX;
    for (; zc > ST_ZC / 2; zc /= 2) {
        long long blocks = 0;
        for (int i = 0; i < n; i++)
            blocks += (long long)((whl[3 * i] + ST_OX - 1) / ST_OX) * ((whl[3 * i + 1] + ST_OY - 1) / ST_OY) *
                      ((whl[3 * i + 2] + zc - 1) / zc);
        if (blocks >= 4LL * 2 * sm_count()) break;
    }
    return zc;
}

int choose_xrpw(const int *whl, int n, int k, int xb_w) {
    const int xt = 32 * xb_w;
    const long long want = 8LL * sm_count();
    int rpw = XP_RPW;
    for (; rpw > 1; rpw /= 2) {
        long long blocks = 0;
        for (int i = 0; i < n; i++) {
            int Wv, Hv, Lv, Wp;
            valid_extents(whl[3 * i], whl[3 * i + 1], whl[3 * i + 2], k, Wv, Hv, Lv, Wp);
            if (Wv > 0)
                blocks += (long long)((Wv + xt - 1) / xt) * ((whl[3 * i + 1] + XP_ROWS * rpw - 1) / (XP_ROWS * rpw)) *
                          whl[3 * i + 2];
        }
        if (blocks >= want) break;
    }
    return rpw;
}

LaunchShape choose_shape(const int *whl, int n, int k, int kspec, int gauss) {
    LaunchShape sh;
    std::vector<int> wv((size_t)n);
    for (int i = 0; i < n; i++) {
        int Wv, Hv, Lv, Wp;
        valid_extents(whl[3 * i], whl[3 * i + 1], whl[3 * i + 2], k, Wv, Hv, Lv, Wp);
        wv[(size_t)i] = Wv;
    }
    sh.xb_w = choose_xb(wv.data(), n);
    sh.xrpw = choose_xrpw(whl, n, k, sh.xb_w);
    sh.pairs = kspec > 0 ? 1 : 0;
    sh.zt = tma_z(kspec) && tma_z_requested() && tensor_maps_available() ? 1 : 0;
    sh.zc = choose_zc(whl, n);
    sh.gauss = gauss;
    return sh;
}

namespace {
// cuTensorMapEncodeTiled from the driver, through the runtime's entry-point
// query (no link against the driver library).
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}
}  // namespace

// The y-pass pair planes as a 4-D float tensor (2 Wp floats, Hv rows, L planes, 2
// pairs); the z-pass box is one plane of a ZT_X x ZT_Y column tile of both
// pairs.  Rows are 8 Wp bytes, a multiple of 32, and the pool offsets keep
// every base 64-byte aligned, as TMA requires.
bool tensor_maps_available() { return tensor_map_encoder() != nullptr; }

// The TMA-fed z-pass runs when the environment variable RSF_ZPASS is "tma"
// (read at each call); the default is the streaming z-pass, which measured
// faster on the 48-sub-volume batch (6.81 against 7.58 ms per launch).
bool tma_z_requested() {
    const char *v = std::getenv("RSF_ZPASS");
    return v && std::strcmp(v, "tma") == 0;
}

bool encode_pair_map(void *out, const SubVolDev &d) {
    static_assert(sizeof(CUtensorMap) == TMAP_BYTES, "tensor map size");
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc || d.Wv <= 0) return false;
    const cuuint64_t dims[4] = {2 * (cuuint64_t)d.Wp, (cuuint64_t)d.Hv, (cuuint64_t)d.L, 2};
    const cuuint64_t row = 8 * (cuuint64_t)d.Wp;
    const cuuint64_t strides[3] = {row, row * d.Hv, row * d.Hv * d.L};
    const cuuint32_t box[4] = {2 * ZT_X, ZT_Y, 1, 2};
    const cuuint32_t estr[4] = {1, 1, 1, 1};
    return enc(static_cast<CUtensorMap *>(out), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, d.yb, dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

void tile_counts(const SubVolDev &d, int kspec, const LaunchShape &sh, int tiles[NPRE]) {
    const bool valid = d.Wv > 0;
    const int xt = 32 * sh.xb_w, zc = sh.zc;
    const int xr = XP_ROWS * sh.xrpw;
    tiles[0] = valid ? ((d.Wv + xt - 1) / xt) * ((d.H + xr - 1) / xr) * d.L : 0;
    if (!valid) tiles[1] = 0;
    else if (kspec == 0) tiles[1] = ((d.Wv + YB_TX - 1) / YB_TX) * ((d.Hv + YB_YB - 1) / YB_YB) * 4 * d.L;
    else tiles[1] = ((d.Wv + YP_COLS - 1) / YP_COLS) * 2 * d.L;  // one column of one pair per thread
    if (!valid) tiles[2] = 0;
    else if (sh.zt) tiles[2] = ((d.Wv + ZT_X - 1) / ZT_X) * ((d.Hv + ZT_Y - 1) / ZT_Y);
    else if (kspec == 0) tiles[2] = ((d.Wv + ZB_TX - 1) / ZB_TX) * ((d.Lv + ZB_ZB - 1) / ZB_ZB) * d.Hv;
    else tiles[2] = ((d.Wv + 2 * ZP_PAIRS - 1) / (2 * ZP_PAIRS)) * d.Hv;
    tiles[3] = ((d.W + ST_OX - 1) / ST_OX) * ((d.H + ST_OY - 1) / ST_OY) * ((d.L + zc - 1) / zc);
    // expanded data term: gauss_x, second y-pass, gauss_z, gauss_border
    const bool g = sh.gauss != 0;
    tiles[NKERN] = g && valid ? ((d.Wv + GX_T * GX_NB - 1) / (GX_T * GX_NB)) * d.H * d.L : 0;
    tiles[NKERN + 1] = g && valid ? ((d.Wv + YB_TX - 1) / YB_TX) * ((d.Hv + YB_YB - 1) / YB_YB) * 4 * d.L : 0;
    tiles[NKERN + 2] = g && valid ? ((d.Wv + ZB_TX - 1) / ZB_TX) * ((d.Lv + ZB_ZB - 1) / ZB_ZB) * d.Hv : 0;
    tiles[NKERN + 3] = g ? (int)(((long long)d.W * d.H * d.L + GB_T - 1) / GB_T) : 0;
}

// Raises the dynamic shared-memory limit of the x-pass instantiations on the
// current device; called once per workspace, outside any stream capture.
cudaError_t configure_device() {
    cudaError_t e = config_xpass_0();
    if (e == cudaSuccess) e = config_xpass_21();
    if (e == cudaSuccess) e = config_xpass_29();
    if (e == cudaSuccess) e = config_xpass_35();
    if (e == cudaSuccess) e = config_ztpass_21();
    if (e == cudaSuccess) e = config_ztpass_35();
    return e;
}

cudaError_t launch_step(const SubVolDev *svs, const int *pre, const int *tot, const StepConst &c, int parity,
                        int arith, unsigned *flag, const DebugOut *dbg, cudaStream_t st, cudaEvent_t *ev) {
    const int n1 = c.nsv + 1;
    const int kspec = kernel_k(c.k, arith, dbg != nullptr, c.box, c.gauss);
    cudaError_t e = cudaSuccess;
    // Inside a stream capture a plain record only orders streams; an external
    // record becomes an event record node of the graph.  Outside a capture
    // the external flag is not allowed.
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (ev && cudaStreamIsCapturing(st, &cap) != cudaSuccess) return cudaGetLastError();
    const unsigned rec_flags = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    auto mark = [&](int i) { return ev ? cudaEventRecordWithFlags(ev[i], st, rec_flags) : cudaSuccess; };
    if ((e = mark(0)) != cudaSuccess) return e;
    if (tot[0] > 0) {
        switch (kspec) {
            case 21: e = launch_xpass_21(svs, pre, tot[0], c, parity, arith, st); break;
            case 29: e = launch_xpass_29(svs, pre, tot[0], c, parity, arith, st); break;
            case 35: e = launch_xpass_35(svs, pre, tot[0], c, parity, arith, st); break;
            default: e = launch_xpass_0(svs, pre, tot[0], c, parity, arith, st); break;
        }
        if (e != cudaSuccess) return e;
    }
    if ((e = mark(1)) != cudaSuccess) return e;
    if (tot[1] > 0) {
        switch (kspec) {
            case 21: e = launch_ypass_21(svs, pre + n1, tot[1], c, st); break;
            case 29: e = launch_ypass_29(svs, pre + n1, tot[1], c, st); break;
            case 35: e = launch_ypass_35(svs, pre + n1, tot[1], c, st); break;
            default: e = launch_ypass_0(svs, pre + n1, tot[1], c, st); break;
        }
        if (e != cudaSuccess) return e;
    }
    if ((e = mark(2)) != cudaSuccess) return e;
    if (tot[2] > 0 && tma_z(kspec) && c.ymaps) {
        e = kspec == 21 ? launch_ztpass_21(svs, pre + 2 * n1, tot[2], c, flag, st)
                        : launch_ztpass_35(svs, pre + 2 * n1, tot[2], c, flag, st);
        if (e != cudaSuccess) return e;
    } else if (tot[2] > 0) {
        switch (kspec) {
            case 21: e = launch_zpass_21(svs, pre + 2 * n1, tot[2], c, dbg, st); break;
            case 29: e = launch_zpass_29(svs, pre + 2 * n1, tot[2], c, dbg, st); break;
            case 35: e = launch_zpass_35(svs, pre + 2 * n1, tot[2], c, dbg, st); break;
            default: e = launch_zpass_0(svs, pre + 2 * n1, tot[2], c, dbg, st); break;
        }
        if (e != cudaSuccess) return e;
    }
    if (c.gauss) {
        e = launch_gauss(svs, pre, n1, tot, c, dbg, st);
        if (e != cudaSuccess) return e;
    }
    if (c.box > 0 && tot[3] > 0) {
        e = launch_box(svs, pre + 3 * n1, tot[3], c, dbg, st);
        if (e != cudaSuccess) return e;
    }
    if ((e = mark(3)) != cudaSuccess) return e;
    if (tot[3] > 0) e = launch_stencil(svs, pre + 3 * n1, tot[3], c, parity, arith, flag, dbg, st);
    if (e == cudaSuccess) e = mark(4);
    return e;
}

}  // namespace rsf
