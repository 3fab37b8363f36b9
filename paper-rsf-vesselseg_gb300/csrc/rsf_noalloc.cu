// rsf_noalloc.cu -- evolution entry point for callers that cannot allocate.
//
// rsf_evolve_noalloc runs the same kernels as rsf_evolve, but every byte of
// scratch (the second level-set buffer, the x- and y-pass fields, the batch
// table and the error flag) lives in one file-scope device array of fixed
// size instead of a caller-created workspace.  It is meant for callers that
// must not allocate device memory once they are running: plug-ins hosted by
// an application that owns the device memory budget through its own pool,
// and real-time loops that forbid allocation after start-up.  The array is
// reserved when this file's module is loaded on a device (with CUDA's
// default lazy loading, at the first call on that device) and is held until
// the process exits.  Its device address is looked up once per device and
// cached, so calls after cudaDeviceReset on that device are not supported.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "rsf.h"
#include "rsf_internal.h"

namespace {

// Largest volume (W*H*L) the static scratch holds.
constexpr int64_t kMaxVoxels = 1 << 20;
// Scratch layout: [table | flag | second phi | x-pass fields | y-pass fields].
constexpr size_t kTableBytes = 4096;
constexpr size_t kFlagBytes = 256;
constexpr size_t kPhiBytes = (size_t)kMaxVoxels * sizeof(float);
constexpr size_t kFieldBytes = 4 * (size_t)kMaxVoxels * sizeof(float);
constexpr size_t kScratchBytes = kTableBytes + kFlagBytes + kPhiBytes + 2 * kFieldBytes;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_ptr[kMaxDevices] = {};

rsf_status fail(rsf_status s, const char *msg) {
    rsf::set_last_error(msg);
    return s;
}

// Device address of the scratch array on the current device.  The host-side
// name g_scratch is not a device address, so it is looked up once per device
// (with that device current) and cached.  The look-up and the kernel
// configuration are not stream work, so a first call made while `st` is
// capturing is refused instead of running them inside the capture.
rsf_status scratch_for_current_device(cudaStream_t st, unsigned char **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return fail(RSF_ERR_NO_DEVICE, "rsf_evolve_noalloc: no usable current CUDA device");
    }
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) {
            cudaGetLastError();
            return fail(RSF_ERR_CUDA, "rsf_evolve_noalloc: cannot query the stream's capture status");
        }
        if (cap != cudaStreamCaptureStatusNone)
            return fail(RSF_ERR_UNSUPPORTED,
                        "rsf_evolve_noalloc: the first call on a device must not be made on a capturing stream");
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || p == nullptr) {
            cudaGetLastError();
            return fail(RSF_ERR_CUDA, "rsf_evolve_noalloc: cudaGetSymbolAddress of the static scratch failed");
        }
        e = rsf::configure_device();
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(RSF_ERR_CUDA, "rsf_evolve_noalloc: kernel configuration failed");
        }
        g_scratch_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_scratch_ptr[dev];
    return RSF_OK;
}

}  // namespace

extern "C" rsf_status rsf_evolve_noalloc(const rsf_params *p, const void *image, rsf_dtype dtype, float *phi,
                                         int64_t W, int64_t H, int64_t L, int32_t iters, void *stream) {
    if (!p || !image || !phi) return fail(RSF_ERR_INVALID_ARGUMENT, "rsf_evolve_noalloc: null argument");
    if (iters < 0) return fail(RSF_ERR_INVALID_ARGUMENT, "rsf_evolve_noalloc: iters must be >= 0");
    if (dtype != RSF_U8 && dtype != RSF_F32) return fail(RSF_ERR_DTYPE, "rsf_evolve_noalloc: dtype must be U8 or F32");
    if (W < 2 || H < 2 || L < 2) return fail(RSF_ERR_SHAPE, "rsf_evolve_noalloc: every extent must be >= 2");
    if (W > kMaxVoxels || H > kMaxVoxels || L > kMaxVoxels || W * H * L > kMaxVoxels)
        return fail(RSF_ERR_WORKSPACE_TOO_SMALL,
                    "rsf_evolve_noalloc: volume exceeds the static scratch limit of 1048576 voxels (W*H*L)");
    const float vals[] = {p->sigma, p->dt, p->mu, p->lambda1, p->lambda2, p->nu, p->eps, p->sigma2};
    for (float v : vals)
        if (!std::isfinite(v)) return fail(RSF_ERR_INVALID_ARGUMENT, "rsf_evolve_noalloc: non-finite parameter");
    if (!(p->eps > 0.0f) || p->sigma2 < 0.0f) return fail(RSF_ERR_INVALID_ARGUMENT, "rsf_evolve_noalloc: bad eps or sigma2");
    if ((int)p->sigma2 != 0) return fail(RSF_ERR_UNSUPPORTED, "rsf_evolve_noalloc: box e-term is not implemented");
    if (p->data_term != RSF_DATA_TERM_REFERENCE)
        return fail(RSF_ERR_UNSUPPORTED, "rsf_evolve_noalloc: the Gaussian data term is not implemented");
    if ((p->boundary != RSF_BOUNDARY_REFERENCE && p->boundary != RSF_BOUNDARY_CLAMP) ||
        (p->arith != RSF_ARITH_PORTABLE && p->arith != RSF_ARITH_REFERENCE))
        return fail(RSF_ERR_INVALID_ARGUMENT, "rsf_evolve_noalloc: unknown boundary or arithmetic mode");
    float taps[rsf::MAXK];
    int k = 0;
    rsf_status s = rsf_gaussian_taps(p->sigma, taps, rsf::MAXK, &k);
    if (s != RSF_OK) return fail(s, "rsf_evolve_noalloc: invalid sigma");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned char *base = nullptr;
    s = scratch_for_current_device(st, &base);
    if (s != RSF_OK) return s;
    if (iters == 0) return RSF_OK;

    rsf::SubVolDev *d_table = reinterpret_cast<rsf::SubVolDev *>(base);
    int *d_pre = reinterpret_cast<int *>(base + 1024);
    unsigned char *d_map = base + 2048;  // TMA map of the y-pass pair planes
    unsigned *d_flag = reinterpret_cast<unsigned *>(base + kTableBytes);
    float *phi2 = reinterpret_cast<float *>(base + kTableBytes + kFlagBytes);
    float *xfields = reinterpret_cast<float *>(base + kTableBytes + kFlagBytes + kPhiBytes);
    float *yfields = reinterpret_cast<float *>(base + kTableBytes + kFlagBytes + kPhiBytes + kFieldBytes);

    rsf::SubVolDev d;
    std::memset(&d, 0, sizeof d);
    d.W = (int)W;
    d.H = (int)H;
    d.L = (int)L;
    rsf::valid_extents(d.W, d.H, d.L, k, d.Wv, d.Hv, d.Lv, d.Wp);
    d.phi[0] = phi;
    d.phi[1] = phi2;
    d.img = image;
    d.xb = xfields;
    d.db = xfields;
    d.yb = yfields;
    const int whl[3] = {d.W, d.H, d.L};
    const int kspec = rsf::kernel_k(k, p->arith, false);
    const rsf::LaunchShape sh = rsf::choose_shape(whl, 1, k, kspec);
    int tiles[rsf::NPRE];
    rsf::tile_counts(d, kspec, sh, tiles);
    int pre[2 * rsf::NPRE];  // per kernel: {0, tiles}
    for (int j = 0; j < rsf::NPRE; j++) {
        pre[2 * j] = 0;
        pre[2 * j + 1] = tiles[j];
    }

    rsf::StepConst c;
    std::memset(&c, 0, sizeof c);
    for (int i = 0; i < k; i++) {
        c.taps[i] = taps[i];
        c.taps2[i] = make_float2(taps[i], taps[i]);
    }
    c.k = k;
    c.r = (k - 1) / 2;
    c.eps = p->eps;
    c.dt = p->dt;
    c.mu = p->mu;
    c.nu = p->nu;
    c.l1 = p->lambda1;
    c.l2 = p->lambda2;
    c.lam_equal = p->lambda1 == p->lambda2;
    c.boundary = p->boundary;
    c.img_f32 = dtype == RSF_F32;
    c.nsv = 1;
    c.xb_w = sh.xb_w;
    c.xrpw = sh.xrpw;
    c.pairs = sh.pairs;
    c.zc = sh.zc;
    alignas(64) unsigned char map[rsf::TMAP_BYTES];
    if (sh.zt) {
        if (!rsf::encode_pair_map(map, d)) return fail(RSF_ERR_CUDA, "rsf_evolve_noalloc: TMA tensor map encoding failed");
        c.ymaps = d_map;
    }

    // The table copies come from pageable host memory: they return once the
    // driver has staged the bytes, so the stack buffers may go out of scope.
    cudaError_t e = cudaMemcpyAsync(d_table, &d, sizeof d, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_pre, pre, sizeof pre, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && sh.zt) e = cudaMemcpyAsync(d_map, map, sizeof map, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_flag, 0, sizeof(unsigned), st);
    for (int it = 0; it < iters && e == cudaSuccess; it++)
        e = rsf::launch_step(d_table, d_pre, tiles, c, it & 1, p->arith, d_flag, nullptr, st);
    if (e == cudaSuccess && (iters & 1))
        e = cudaMemcpyAsync(phi, phi2, (size_t)W * H * L * sizeof(float), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
        char msg[256];
        std::snprintf(msg, sizeof msg, "rsf_evolve_noalloc: %s", cudaGetErrorString(e));
        return fail(RSF_ERR_CUDA, msg);
    }
    return RSF_OK;
}
