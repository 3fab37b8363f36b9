// rsf_capi.cu -- the extern "C" boundary declared in include/rsf.h.
//
// Replaces the reference's host layer: the per-op wrappers of
// CUDA_RSF/kernel.cu (each a cudaMalloc / cudaMemcpy / launch / cudaMemcpy /
// cudaFree bracket, forward-declared at CUDA_RSF/main.cpp:56-71) and the
// iteration loop of CUDA_RSF/main.cpp:222-314.  Here the state stays resident
// in device memory, scratch lives in a caller-owned workspace, and a batch of
// sub-volumes advances one iteration per four kernel launches (x-pass, y-pass,
// z-pass, stencil/update).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "rsf.h"
#include "rsf_internal.h"

using rsf::StepConst;
using rsf::SubVolDev;

namespace {
thread_local char g_last_error[512] = "";

rsf_status cuda_fail(cudaError_t e, const char *what) {
    std::snprintf(g_last_error, sizeof g_last_error, "%s: %s", what, cudaGetErrorString(e));
    return RSF_ERR_CUDA;
}

rsf_status fail(rsf_status s, const char *msg) {
    std::snprintf(g_last_error, sizeof g_last_error, "%s", msg);
    return s;
}

constexpr int64_t kMaxExtent = 1 << 20;
}  // namespace

void rsf::set_last_error(const char *msg) { std::snprintf(g_last_error, sizeof g_last_error, "%s", msg); }

struct rsf_workspace {
    int device = -1;
    int64_t max_voxels = 0;
    int32_t max_subvols = 0;
    float *pool_phi2 = nullptr;  // second level-set buffer, max_voxels
    float *pool_x = nullptr;     // x-pass fields, 4 * max_voxels
    float *pool_y = nullptr;     // y-pass fields, 4 * max_voxels
    float *pool_g = nullptr;     // expanded data term's x-blurred fields, 4 * max_voxels (first use)
    SubVolDev *d_svs = nullptr;
    int *d_pre = nullptr;        // NPRE * (max_subvols + 1)
    unsigned char *d_maps = nullptr;  // TMA maps of the pair planes, max_subvols * TMAP_BYTES
    unsigned *d_flag = nullptr;
    // Pinned staging of the table, kStages slots used in turn: a call waits
    // only for the upload of the call kStages before it, so consecutive
    // calls do not make the host wait for the device.
    static constexpr int kStages = 4;
    SubVolDev *h_svs = nullptr;  // kStages * max_subvols
    int *h_pre = nullptr;        // kStages * NPRE * (max_subvols + 1)
    unsigned char *h_maps = nullptr;  // kStages * max_subvols * TMAP_BYTES
    rsf::AdjVol *h_adj = nullptr;     // kStages * max_subvols (adjoint batches)
    int *h_adj_pre = nullptr;         // kStages * NADJ * (max_subvols + 1)
    rsf::AdjVol *d_adj = nullptr;
    int *d_adj_pre = nullptr;
    cudaEvent_t table_ev[kStages] = {};
    bool table_pending[kStages] = {};
    int stage = 0;
    // Staging slot for the next upload; waits until its previous upload is done.
    cudaError_t next_stage(SubVolDev **svs, int **pre, unsigned char **maps) {
        if (table_pending[stage]) {
            cudaError_t e = cudaEventSynchronize(table_ev[stage]);
            if (e != cudaSuccess) return e;
            table_pending[stage] = false;
        }
        *svs = h_svs + (size_t)stage * max_subvols;
        *pre = h_pre + (size_t)stage * rsf::NPRE * ((size_t)max_subvols + 1);
        *maps = h_maps + (size_t)stage * max_subvols * rsf::TMAP_BYTES;
        return cudaSuccess;
    }
    int current_stage() const { return stage; }
    cudaError_t mark_stage(cudaStream_t st) {
        cudaError_t e = cudaEventRecord(table_ev[stage], st);
        if (e == cudaSuccess) {
            table_pending[stage] = true;
            stage = (stage + 1) % kStages;
        }
        return e;
    }
    cudaStream_t capture_stream = nullptr;
    size_t bytes = 0;
    // launch-shape overrides (rsf_workspace_set_launch_shape; 0 / -1: automatic)
    int force_xb = 0, force_zc = 0, force_zt = -1;
    // host-buffer convenience path (allocated on first use)
    void *stage_img = nullptr;
    float *stage_phi = nullptr;
    size_t stage_voxels = 0;
    // per-kernel timing (rsf_set_kernel_timing): events between launches
    bool timing = false;
    std::vector<cudaEvent_t> events;
    int pending_iters = 0;            // iterations whose events are not read yet
    int pending_tot[rsf::NKERN] = {0, 0, 0, 0};
    double kernel_ms[rsf::NKERN] = {0, 0, 0, 0};
    long long kernel_launches[rsf::NKERN] = {0, 0, 0, 0};
};

namespace {
// The address through which the device reads or writes `ptr`: the pointer
// itself for device or managed memory, the mapped address for pinned or
// registered host memory, null for pageable host memory.
void *device_view(const void *ptr) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeHost || a.type == cudaMemoryTypeManaged)
        return a.devicePointer;
    return nullptr;
}

// Host <-> device staging copy: SM copy when the host side is pinned, else
// the copy engine (pageable memory).
cudaError_t stage_copy(void *dst, const void *src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st) {
    const bool h2d = kind == cudaMemcpyHostToDevice;
    void *hv = device_view(h2d ? src : dst);
    if (hv) return h2d ? rsf::launch_copy(dst, hv, bytes, st) : rsf::launch_copy(hv, src, bytes, st);
    return cudaMemcpyAsync(dst, src, bytes, kind, st);
}
}  // namespace

extern "C" {

int rsf_abi_version(void) { return RSF_ABI_VERSION; }

const char *rsf_last_error(void) { return g_last_error; }

const char *rsf_status_string(rsf_status s) {
    switch (s) {
        case RSF_OK: return "ok";
        case RSF_ERR_INVALID_ARGUMENT: return "invalid argument";
        case RSF_ERR_SHAPE: return "invalid volume shape";
        case RSF_ERR_DTYPE: return "unsupported image dtype";
        case RSF_ERR_UNSUPPORTED: return "unsupported parameter combination";
        case RSF_ERR_NO_MEMORY: return "device memory allocation failed";
        case RSF_ERR_WORKSPACE_TOO_SMALL: return "workspace too small for this batch";
        case RSF_ERR_CUDA: return "CUDA runtime error";
        case RSF_ERR_NONFINITE: return "non-finite value in the level set";
        case RSF_ERR_IO: return "file input/output error";
        case RSF_ERR_NO_DEVICE: return "no CUDA device";
    }
    return "unknown status";
}

rsf_status rsf_params_default(rsf_params *p) {
    if (!p) return fail(RSF_ERR_INVALID_ARGUMENT, "params is null");
    std::memset(p, 0, sizeof *p);
    p->sigma = 5.0f;
    p->dt = 0.1f;
    p->mu = 1.0f;
    p->lambda1 = 0.1f;
    p->lambda2 = 0.1f;
    p->nu = 0.0001f;
    p->eps = 0.2f;
    p->sigma2 = 0.0f;
    p->boundary = RSF_BOUNDARY_REFERENCE;
    p->arith = RSF_ARITH_PORTABLE;
    return RSF_OK;
}

// CUDA_RSF/main.cpp:152-166.  exp is evaluated in double and rounded so that
// the taps are the same on every host.
rsf_status rsf_gaussian_taps(float sigma, float *taps, int cap, int *k_out) {
    if (!(sigma > 0.0f) || !std::isfinite(sigma)) return fail(RSF_ERR_INVALID_ARGUMENT, "sigma must be > 0");
    const float p7 = 7.0f * sigma;
    if (p7 > (float)(rsf::MAXK)) return fail(RSF_ERR_UNSUPPORTED, "sigma too large (more than 128 taps)");
    unsigned p = (unsigned)p7;
    if (p % 2u == 0u) p++;
    const float miu = (float)(p / 2u);
    const int u = (int)(2.0f * sigma * sigma);
    if (u < 1) return fail(RSF_ERR_INVALID_ARGUMENT, "sigma too small: (int)(2 sigma^2) must be >= 1");
    if ((int)p > rsf::MAXK) return fail(RSF_ERR_UNSUPPORTED, "more than 128 taps");
    if (k_out) *k_out = (int)p;
    if (!taps) return RSF_OK;
    if (cap < (int)p) return fail(RSF_ERR_INVALID_ARGUMENT, "taps buffer too small");
    const float s = std::sqrt((float)u * (float)3.14159265358979323846);
    for (unsigned xi = 0; xi < p; xi++) {
        const float d = (float)(int)xi - miu;
        const float a = (-d * d) / (float)u;
        taps[xi] = (1.0f / s) * (float)std::exp((double)a);
    }
    return RSF_OK;
}

size_t rsf_workspace_bytes_for(int64_t max_voxels, int32_t max_subvols) {
    const size_t v = (size_t)std::max<int64_t>(max_voxels, 0);
    const size_t n = (size_t)std::max<int32_t>(max_subvols, 1);
    return v * sizeof(float) * 9 + n * (sizeof(SubVolDev) + rsf::TMAP_BYTES + sizeof(rsf::AdjVol)) +
           (rsf::NPRE + rsf::NADJ) * (n + 1) * sizeof(int) + 256;
}

static void ws_free(rsf_workspace *ws) {
    if (!ws) return;
    int cur = -1;
    cudaGetDevice(&cur);
    if (ws->device >= 0) cudaSetDevice(ws->device);
    for (cudaEvent_t ev : ws->table_ev)
        if (ev) cudaEventSynchronize(ev);
    cudaFree(ws->pool_phi2);
    cudaFree(ws->pool_x);
    cudaFree(ws->pool_y);
    cudaFree(ws->pool_g);
    cudaFree(ws->d_svs);
    cudaFree(ws->d_pre);
    cudaFree(ws->d_maps);
    cudaFree(ws->d_adj);
    cudaFree(ws->d_adj_pre);
    cudaFree(ws->d_flag);
    cudaFree(ws->stage_img);
    cudaFree(ws->stage_phi);
    cudaFreeHost(ws->h_svs);
    cudaFreeHost(ws->h_pre);
    cudaFreeHost(ws->h_maps);
    cudaFreeHost(ws->h_adj);
    cudaFreeHost(ws->h_adj_pre);
    for (cudaEvent_t ev : ws->table_ev)
        if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : ws->events) cudaEventDestroy(ev);
    if (ws->capture_stream) cudaStreamDestroy(ws->capture_stream);
    if (cur >= 0) cudaSetDevice(cur);
    delete ws;
}

rsf_status rsf_workspace_create(int64_t max_voxels, int32_t max_subvols, rsf_workspace **out) {
    if (!out) return fail(RSF_ERR_INVALID_ARGUMENT, "output pointer is null");
    *out = nullptr;
    if (max_voxels < 1 || max_subvols < 1) return fail(RSF_ERR_INVALID_ARGUMENT, "max_voxels and max_subvols must be >= 1");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        return fail(RSF_ERR_NO_DEVICE, "no CUDA device visible");
    }
    rsf_workspace *ws = new rsf_workspace;
    cudaGetDevice(&ws->device);
    ws->max_voxels = max_voxels;
    ws->max_subvols = max_subvols;
    const size_t v = (size_t)max_voxels;
    cudaError_t e = cudaSuccess;
    auto alloc = [&](void **p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    };
    alloc((void **)&ws->pool_phi2, v * sizeof(float));
    alloc((void **)&ws->pool_x, 4 * v * sizeof(float));
    alloc((void **)&ws->pool_y, 4 * v * sizeof(float));
    alloc((void **)&ws->d_svs, (size_t)max_subvols * sizeof(SubVolDev));
    alloc((void **)&ws->d_pre, rsf::NPRE * ((size_t)max_subvols + 1) * sizeof(int));
    alloc((void **)&ws->d_maps, (size_t)max_subvols * rsf::TMAP_BYTES);
    alloc((void **)&ws->d_adj, (size_t)max_subvols * sizeof(rsf::AdjVol));
    alloc((void **)&ws->d_adj_pre, rsf::NADJ * ((size_t)max_subvols + 1) * sizeof(int));
    alloc((void **)&ws->d_flag, 256);
    const size_t ns = rsf_workspace::kStages;
    if (e == cudaSuccess) e = cudaMallocHost((void **)&ws->h_svs, ns * (size_t)max_subvols * sizeof(SubVolDev));
    if (e == cudaSuccess)
        e = cudaMallocHost((void **)&ws->h_pre, ns * rsf::NPRE * ((size_t)max_subvols + 1) * sizeof(int));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&ws->h_maps, ns * (size_t)max_subvols * rsf::TMAP_BYTES);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&ws->h_adj, ns * (size_t)max_subvols * sizeof(rsf::AdjVol));
    if (e == cudaSuccess)
        e = cudaMallocHost((void **)&ws->h_adj_pre, ns * rsf::NADJ * ((size_t)max_subvols + 1) * sizeof(int));
    for (size_t i = 0; i < ns && e == cudaSuccess; i++)
        e = cudaEventCreateWithFlags(&ws->table_ev[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ws->capture_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMemset(ws->d_flag, 0, 256);
    if (e == cudaSuccess) e = rsf::configure_device();
    if (e != cudaSuccess) {
        const bool oom = e == cudaErrorMemoryAllocation;
        cudaGetLastError();
        ws_free(ws);
        return oom ? fail(RSF_ERR_NO_MEMORY, "workspace allocation failed") : cuda_fail(e, "workspace create");
    }
    ws->bytes = rsf_workspace_bytes_for(max_voxels, max_subvols);
    *out = ws;
    return RSF_OK;
}

rsf_status rsf_workspace_destroy(rsf_workspace *ws) {
    if (!ws) return fail(RSF_ERR_INVALID_ARGUMENT, "workspace is null");
    ws_free(ws);
    return RSF_OK;
}

size_t rsf_workspace_bytes(const rsf_workspace *ws) { return ws ? ws->bytes : 0; }

rsf_status rsf_workspace_set_launch_shape(rsf_workspace *ws, int32_t xpass_width, int32_t stencil_planes,
                                          int32_t z_tma) {
    if (!ws) return fail(RSF_ERR_INVALID_ARGUMENT, "workspace is null");
    if (xpass_width != 0 && xpass_width != rsf::XB_CHOICES[0] && xpass_width != rsf::XB_CHOICES[1])
        return fail(RSF_ERR_INVALID_ARGUMENT, "x-pass width must be 0 (automatic), 5 or 9");
    if (stencil_planes != 0 && stencil_planes != rsf::ST_ZC_MAX && stencil_planes != rsf::ST_ZC &&
        stencil_planes != rsf::ST_ZC / 2)
        return fail(RSF_ERR_INVALID_ARGUMENT, "stencil planes must be 0 (automatic), 32, 64 or 128");
    if (z_tma < -1 || z_tma > 1) return fail(RSF_ERR_INVALID_ARGUMENT, "z_tma must be -1 (automatic), 0 or 1");
    ws->force_xb = xpass_width;
    ws->force_zc = stencil_planes;
    ws->force_zt = z_tma;
    return RSF_OK;
}

}  // extern "C"

namespace {

rsf_status check_params(const rsf_params *p, int *k, float *taps) {
    if (!p) return fail(RSF_ERR_INVALID_ARGUMENT, "params is null");
    const float vals[] = {p->sigma, p->dt, p->mu, p->lambda1, p->lambda2, p->nu, p->eps, p->sigma2};
    for (float v : vals)
        if (!std::isfinite(v)) return fail(RSF_ERR_INVALID_ARGUMENT, "non-finite parameter");
    if (!(p->eps > 0.0f)) return fail(RSF_ERR_INVALID_ARGUMENT, "eps must be > 0");
    if (p->sigma2 < 0.0f) return fail(RSF_ERR_INVALID_ARGUMENT, "sigma2 must be >= 0");
    if (p->sigma2 >= (float)(rsf::MAX_BOX + 1)) return fail(RSF_ERR_UNSUPPORTED, "sigma2 above 8 is not supported");
    if (p->boundary != RSF_BOUNDARY_REFERENCE && p->boundary != RSF_BOUNDARY_CLAMP)
        return fail(RSF_ERR_INVALID_ARGUMENT, "unknown boundary mode");
    if (p->arith != RSF_ARITH_PORTABLE && p->arith != RSF_ARITH_REFERENCE)
        return fail(RSF_ERR_INVALID_ARGUMENT, "unknown arithmetic mode");
    if (p->data_term != RSF_DATA_TERM_REFERENCE && p->data_term != RSF_DATA_TERM_GAUSSIAN)
        return fail(RSF_ERR_INVALID_ARGUMENT, "unknown data term");
    if (p->data_term == RSF_DATA_TERM_GAUSSIAN && p->sigma2 >= 1.0f)
        return fail(RSF_ERR_UNSUPPORTED, "the Gaussian data term takes no box window (sigma2 < 1)");
    return rsf_gaussian_taps(p->sigma, taps, rsf::MAXK, k);
}

rsf_status check_shape(int64_t W, int64_t H, int64_t L) {
    if (W < 2 || H < 2 || L < 2) return fail(RSF_ERR_SHAPE, "every extent must be >= 2");
    if (W > kMaxExtent || H > kMaxExtent || L > kMaxExtent) return fail(RSF_ERR_SHAPE, "extent too large");
    if ((double)W * (double)H * (double)L > 1.0e12) return fail(RSF_ERR_SHAPE, "volume too large");
    return RSF_OK;
}

// Lays out a batch in the workspace pools and uploads the table.
rsf_status prepare(rsf_workspace *ws, const rsf_subvol *svs, int32_t n, int k, int kspec, int box, int gauss,
                   rsf_dtype dtype, const float *const *phi_out_override, int totals[rsf::NPRE],
                   rsf::LaunchShape *shape, cudaStream_t st) {
    const bool full_data = box > 0 || gauss;
    if (n < 1) return fail(RSF_ERR_INVALID_ARGUMENT, "batch is empty");
    if (n > ws->max_subvols) return fail(RSF_ERR_WORKSPACE_TOO_SMALL, "more sub-volumes than the workspace holds");
    if (dtype != RSF_U8 && dtype != RSF_F32) return fail(RSF_ERR_DTYPE, "image dtype must be RSF_U8 or RSF_F32");
    int64_t total = 0;
    for (int i = 0; i < n; i++) {
        if (!svs[i].phi || !svs[i].image) return fail(RSF_ERR_INVALID_ARGUMENT, "null sub-volume pointer");
        rsf_status s = check_shape(svs[i].W, svs[i].H, svs[i].L);
        if (s != RSF_OK) return s;
        total += svs[i].W * svs[i].H * svs[i].L;
    }
    if (total > ws->max_voxels) return fail(RSF_ERR_WORKSPACE_TOO_SMALL, "batch larger than the workspace");
    SubVolDev *h_svs = nullptr;
    int *h_pre = nullptr;
    unsigned char *h_maps = nullptr;
    {
        cudaError_t e = ws->next_stage(&h_svs, &h_pre, &h_maps);
        if (e != cudaSuccess) return cuda_fail(e, "table event");
    }
    std::vector<int> whl(3 * (size_t)n);
    for (int i = 0; i < n; i++) {
        whl[3 * i] = (int)svs[i].W;
        whl[3 * i + 1] = (int)svs[i].H;
        whl[3 * i + 2] = (int)svs[i].L;
    }
    *shape = rsf::choose_shape(whl.data(), n, k, kspec, gauss);
    if (ws->force_xb) {
        shape->xb_w = ws->force_xb;
        shape->xrpw = rsf::choose_xrpw(whl.data(), n, k, shape->xb_w);
    }
    if (ws->force_zc) shape->zc = ws->force_zc;
    if (ws->force_zt >= 0) shape->zt = ws->force_zt && rsf::tma_z(kspec) && rsf::tensor_maps_available() ? 1 : 0;
    const int n1 = n + 1;
    int *pre = h_pre;
    for (int j = 0; j < rsf::NPRE; j++) pre[j * n1] = 0;
    size_t off_v = 0, off_x = 0, off_y = 0;
    for (int i = 0; i < n; i++) {
        SubVolDev d;
        std::memset(&d, 0, sizeof d);
        d.W = (int)svs[i].W;
        d.H = (int)svs[i].H;
        d.L = (int)svs[i].L;
        rsf::valid_extents(d.W, d.H, d.L, k, d.Wv, d.Hv, d.Lv, d.Wp);
        int tiles[rsf::NPRE];
        rsf::tile_counts(d, kspec, *shape, tiles);
        const size_t nv = (size_t)d.W * d.H * d.L;
        d.phi[0] = svs[i].phi;
        d.phi[1] = phi_out_override ? const_cast<float *>(phi_out_override[i]) : ws->pool_phi2 + off_v;
        d.img = svs[i].image;
        d.xb = ws->pool_x + off_x;
        d.db = d.xb;  // the data factor reuses the x-pass storage
        d.yb = ws->pool_y + off_y;
        off_v += nv;
        // x-pass slot: the four x-pass fields, or with the box e-term or the
        // expanded data term f_out, f_in of the valid region followed by the
        // data factor of every voxel (the expanded term's blurred fields use
        // the same offsets in pool_g)
        // (rounded up to 4 floats for the vector accesses).  Both are at most
        // 4 W H L floats (Wp < W since k >= 5), so the pool of 4 max_voxels
        // floats holds every batch that passes the voxel check above.
        size_t slot_x = 4 * (size_t)d.Wp * d.H * d.L;
        if (full_data) slot_x = std::max(slot_x, (2 * (size_t)d.Wp * d.Hv * d.Lv + nv + 3) & ~(size_t)3);
        off_x += slot_x;
        off_y += 4 * (size_t)d.Wp * d.Hv * d.L;
        for (int j = 0; j < rsf::NPRE; j++) {
            const int64_t next = (int64_t)pre[j * n1 + i] + tiles[j];
            if (next > 0x7fffffffLL) return fail(RSF_ERR_SHAPE, "batch needs more than 2^31 blocks");
            pre[j * n1 + i + 1] = (int)next;
        }
        h_svs[i] = d;
        if (shape->zt && d.Wv > 0 && !rsf::encode_pair_map(h_maps + (size_t)i * rsf::TMAP_BYTES, d))
            return fail(RSF_ERR_CUDA, "TMA tensor map encoding of the pair planes failed");
    }
    for (int j = 0; j < rsf::NPRE; j++) totals[j] = pre[j * n1 + n];
    cudaError_t e = cudaMemcpyAsync(ws->d_svs, h_svs, (size_t)n * sizeof(SubVolDev), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ws->d_pre, h_pre, rsf::NPRE * (size_t)n1 * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && shape->zt)
        e = cudaMemcpyAsync(ws->d_maps, h_maps, (size_t)n * rsf::TMAP_BYTES, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = ws->mark_stage(st);
    if (e != cudaSuccess) return cuda_fail(e, "table upload");
    return RSF_OK;
}

StepConst make_const(const rsf_params *p, int k, const float *taps, rsf_dtype dtype, int n,
                     const rsf::LaunchShape &sh, const void *maps) {
    StepConst c;
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
    c.nsv = n;
    c.xb_w = sh.xb_w;
    c.xrpw = sh.xrpw;
    c.pairs = sh.pairs;
    c.zc = sh.zc;
    c.ymaps = sh.zt ? maps : nullptr;
    c.box = (int)p->sigma2;
    c.gauss = p->data_term == RSF_DATA_TERM_GAUSSIAN;
    c.full_data = c.box > 0 || c.gauss;
    // K*1: the valid correlation of ones in the blur's own order (fused
    // multiply-adds from +0 over ascending taps, x, then y, then z)
    float sx = 0.0f, sy = 0.0f, s3 = 0.0f;
    for (int i = 0; i < k; i++) sx = std::fma(1.0f, taps[i], sx);
    for (int i = 0; i < k; i++) sy = std::fma(sx, taps[i], sy);
    for (int i = 0; i < k; i++) s3 = std::fma(sy, taps[i], s3);
    c.s3 = s3;
    c.gdelta = 0;
    return c;
}

// The expanded data term's scratch (4 floats per voxel of the workspace's
// capacity), allocated on its first use; returns the offset of its slots
// from the x-pass pool's.
rsf_status gauss_pool(rsf_workspace *ws, ptrdiff_t *delta) {
    if (!ws->pool_g) {
        cudaError_t e = cudaMalloc((void **)&ws->pool_g, 4 * (size_t)ws->max_voxels * sizeof(float));
        if (e != cudaSuccess) {
            cudaGetLastError();
            ws->pool_g = nullptr;
            return fail(RSF_ERR_NO_MEMORY, "allocation of the Gaussian data term's scratch failed");
        }
        ws->bytes += 4 * (size_t)ws->max_voxels * sizeof(float);
    }
    *delta = ws->pool_g - ws->pool_x;
    return RSF_OK;
}

// Copies the second buffer back into the caller's phi after an odd number
// of iterations.
rsf_status copy_back(rsf_workspace *ws, const rsf_subvol *svs, int32_t n, cudaStream_t st) {
    size_t off = 0;
    for (int i = 0; i < n; i++) {
        const size_t nv = (size_t)svs[i].W * svs[i].H * svs[i].L;
        cudaError_t e = cudaMemcpyAsync(svs[i].phi, ws->pool_phi2 + off, nv * sizeof(float), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_fail(e, "copy back");
        off += nv;
    }
    return RSF_OK;
}

// Reads the events of the last timed evolution into the per-kernel totals.
rsf_status collect_times(rsf_workspace *ws) {
    if (ws->pending_iters == 0) return RSF_OK;
    cudaError_t e = cudaEventSynchronize(ws->events[(size_t)rsf::NKERN * ws->pending_iters]);
    if (e != cudaSuccess) return cuda_fail(e, "timing events");
    for (int it = 0; it < ws->pending_iters; it++)
        for (int j = 0; j < rsf::NKERN; j++) {
            float ms = 0.0f;
            e = cudaEventElapsedTime(&ms, ws->events[(size_t)rsf::NKERN * it + j],
                                     ws->events[(size_t)rsf::NKERN * it + j + 1]);
            if (e != cudaSuccess) return cuda_fail(e, "timing events");
            ws->kernel_ms[j] += ms;
            if (ws->pending_tot[j] > 0) ws->kernel_launches[j]++;
        }
    ws->pending_iters = 0;
    return RSF_OK;
}

// Events for `iters` timed iterations: NKERN per iteration plus one, each
// iteration's last event being the next one's first.
rsf_status timing_events(rsf_workspace *ws, int iters, const int tot[rsf::NKERN]) {
    rsf_status s = collect_times(ws);
    if (s != RSF_OK) return s;
    const size_t need = (size_t)rsf::NKERN * iters + 1;
    while (ws->events.size() < need) {
        cudaEvent_t ev;
        cudaError_t e = cudaEventCreate(&ev);
        if (e != cudaSuccess) return cuda_fail(e, "event create");
        ws->events.push_back(ev);
    }
    ws->pending_iters = iters;
    for (int j = 0; j < rsf::NKERN; j++) ws->pending_tot[j] = tot[j];
    return RSF_OK;
}

rsf_status run(rsf_workspace *ws, const rsf_params *p, rsf_dtype dtype, const rsf_subvol *svs, int32_t n,
               int32_t iters, cudaStream_t st, bool use_graph) {
    if (!ws) return fail(RSF_ERR_INVALID_ARGUMENT, "workspace is null");
    if (iters < 0) return fail(RSF_ERR_INVALID_ARGUMENT, "iters must be >= 0");
    float taps[rsf::MAXK];
    int k = 0;
    rsf_status s = check_params(p, &k, taps);
    if (s != RSF_OK) return s;
    int tot[rsf::NPRE];
    rsf::LaunchShape sh;
    const int gauss = p->data_term == RSF_DATA_TERM_GAUSSIAN;
    s = prepare(ws, svs, n, k, rsf::kernel_k(k, p->arith, false, (int)p->sigma2, gauss), (int)p->sigma2, gauss, dtype,
                nullptr, tot, &sh, st);
    if (s != RSF_OK) return s;
    if (iters == 0) return RSF_OK;
    StepConst c = make_const(p, k, taps, dtype, n, sh, ws->d_maps);
    if (gauss && (s = gauss_pool(ws, &c.gdelta)) != RSF_OK) return s;
    if (ws->timing) {
        s = timing_events(ws, iters, tot);
        if (s != RSF_OK) return s;
    }
    auto step = [&](int it, cudaStream_t on) {
        cudaEvent_t *ev = ws->timing ? &ws->events[(size_t)rsf::NKERN * it] : nullptr;
        return rsf::launch_step(ws->d_svs, ws->d_pre, tot, c, it & 1, p->arith, ws->d_flag, nullptr, on, ev);
    };
    cudaError_t e = cudaSuccess;
    if (!use_graph) {
        for (int it = 0; it < iters && e == cudaSuccess; it++) e = step(it, st);
        if (e != cudaSuccess) return cuda_fail(e, "step launch");
    } else {
        // Capture iterations [first, first + count) into one executable graph.
        auto capture = [&](int first, int count, cudaGraphExec_t *exec) -> cudaError_t {
            cudaGraph_t g = nullptr;
            cudaError_t err = cudaStreamBeginCapture(ws->capture_stream, cudaStreamCaptureModeThreadLocal);
            if (err != cudaSuccess) return err;
            for (int it = first; it < first + count && err == cudaSuccess; it++) err = step(it, ws->capture_stream);
            cudaError_t end = cudaStreamEndCapture(ws->capture_stream, &g);
            if (err == cudaSuccess) err = end;
            if (err == cudaSuccess) err = cudaGraphInstantiate(exec, g, 0);
            if (g) cudaGraphDestroy(g);
            return err;
        };
        if (ws->timing) {
            // every iteration has its own events: capture the whole evolution
            cudaGraphExec_t all = nullptr;
            e = capture(0, iters, &all);
            if (e == cudaSuccess) e = cudaGraphLaunch(all, st);
            if (all) cudaGraphExecDestroy(all);
        } else {
            // two iterations (phi -> phi2 -> phi) captured once and replayed
            cudaGraphExec_t pair = nullptr, single = nullptr;
            if (iters >= 2) e = capture(0, 2, &pair);
            if (e == cudaSuccess && (iters & 1)) e = capture(0, 1, &single);
            for (int i = 0; i < iters / 2 && e == cudaSuccess; i++) e = cudaGraphLaunch(pair, st);
            if (e == cudaSuccess && single) e = cudaGraphLaunch(single, st);
            if (pair) cudaGraphExecDestroy(pair);
            if (single) cudaGraphExecDestroy(single);
        }
        if (e != cudaSuccess) return cuda_fail(e, "graph");
    }
    if (iters & 1) return copy_back(ws, svs, n, st);
    return RSF_OK;
}

}  // namespace

extern "C" {

rsf_status rsf_evolve(rsf_workspace *ws, const rsf_params *p, const void *image, rsf_dtype dtype, float *phi,
                      int64_t W, int64_t H, int64_t L, int32_t iters, void *stream) {
    rsf_subvol sv = {phi, image, W, H, L};
    return run(ws, p, dtype, &sv, 1, iters, (cudaStream_t)stream, false);
}

rsf_status rsf_evolve_batched(rsf_workspace *ws, const rsf_params *p, rsf_dtype dtype, const rsf_subvol *subvols,
                              int32_t n, int32_t iters, void *stream) {
    if (!subvols) return fail(RSF_ERR_INVALID_ARGUMENT, "subvols is null");
    return run(ws, p, dtype, subvols, n, iters, (cudaStream_t)stream, true);
}

rsf_status rsf_evolve_host(rsf_workspace *ws, const rsf_params *p, const void *image_host, rsf_dtype dtype,
                           float *phi_host, int64_t W, int64_t H, int64_t L, int32_t iters) {
    if (!ws || !image_host || !phi_host) return fail(RSF_ERR_INVALID_ARGUMENT, "null argument");
    rsf_status s = check_shape(W, H, L);
    if (s != RSF_OK) return s;
    if (dtype != RSF_U8 && dtype != RSF_F32) return fail(RSF_ERR_DTYPE, "image dtype must be RSF_U8 or RSF_F32");
    const size_t nv = (size_t)W * H * L;
    if ((int64_t)nv > ws->max_voxels) return fail(RSF_ERR_WORKSPACE_TOO_SMALL, "volume larger than the workspace");
    if (ws->stage_voxels < nv) {
        cudaFree(ws->stage_img);
        cudaFree(ws->stage_phi);
        ws->stage_img = nullptr;
        ws->stage_phi = nullptr;
        ws->stage_voxels = 0;
        cudaError_t e = cudaMalloc(&ws->stage_img, nv * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc((void **)&ws->stage_phi, nv * sizeof(float));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return fail(RSF_ERR_NO_MEMORY, "staging allocation failed");
        }
        ws->stage_voxels = nv;
    }
    const size_t ib = nv * (dtype == RSF_F32 ? 4 : 1);
    cudaStream_t st = ws->capture_stream;
    cudaError_t e = stage_copy(ws->stage_img, image_host, ib, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = stage_copy(ws->stage_phi, phi_host, nv * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "host to device");
    rsf_subvol sv = {ws->stage_phi, ws->stage_img, W, H, L};
    s = run(ws, p, dtype, &sv, 1, iters, st, false);
    if (s != RSF_OK) return s;
    e = stage_copy(phi_host, ws->stage_phi, nv * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "device to host");
    return RSF_OK;
}

rsf_status rsf_step_debug(rsf_workspace *ws, const rsf_params *p, const void *image, rsf_dtype dtype,
                          const float *phi, float *phi_out, float *fields, int64_t W, int64_t H, int64_t L,
                          void *stream) {
    if (!ws || !phi || !phi_out || !fields || !image) return fail(RSF_ERR_INVALID_ARGUMENT, "null argument");
    float taps[rsf::MAXK];
    int k = 0;
    rsf_status s = check_params(p, &k, taps);
    if (s != RSF_OK) return s;
    rsf_subvol sv = {const_cast<float *>(phi), image, W, H, L};
    const float *outs[1] = {phi_out};
    int tot[rsf::NPRE];
    rsf::LaunchShape sh;
    cudaStream_t st = (cudaStream_t)stream;
    const int gauss = p->data_term == RSF_DATA_TERM_GAUSSIAN;
    s = prepare(ws, &sv, 1, k, rsf::kernel_k(k, p->arith, true), (int)p->sigma2, gauss, dtype, outs, tot, &sh, st);
    if (s != RSF_OK) return s;
    StepConst c = make_const(p, k, taps, dtype, 1, sh, ws->d_maps);
    if (gauss && (s = gauss_pool(ws, &c.gdelta)) != RSF_OK) return s;
    const rsf::DebugOut dbg = {fields, (int64_t)W * H * L};
    cudaError_t e = rsf::launch_step(ws->d_svs, ws->d_pre, tot, c, 0, p->arith, ws->d_flag, &dbg, st);
    return e == cudaSuccess ? RSF_OK : cuda_fail(e, "debug step");
}

// CUDA_RSF/main.cpp:174-183: phi0 = sdf(seed - 13).  The transform is defined
// in rsf_sdf.cu; scratch is the x-field pool (12 of its 16 bytes per voxel).
rsf_status rsf_signed_distance(rsf_workspace *ws, const void *seed, rsf_dtype dtype, float threshold, float *phi,
                               int64_t W, int64_t H, int64_t L, void *stream) {
    if (!ws) return fail(RSF_ERR_INVALID_ARGUMENT, "workspace is null");
    if (!seed || !phi) return fail(RSF_ERR_INVALID_ARGUMENT, "seed and phi must be device pointers");
    if (dtype != RSF_U8 && dtype != RSF_F32) return fail(RSF_ERR_DTYPE, "seed dtype must be RSF_U8 or RSF_F32");
    if (W < 1 || H < 1 || L < 1) return fail(RSF_ERR_SHAPE, "W, H and L must be >= 1");
    if (W > 32768 || H > 32768 || L > 32768) return fail(RSF_ERR_SHAPE, "extents above 32768 are not supported");
    const uint64_t dmax = (uint64_t)(W - 1) * (W - 1) + (uint64_t)(H - 1) * (H - 1) + (uint64_t)(L - 1) * (L - 1);
    if (dmax >= 0xffffffffull) return fail(RSF_ERR_SHAPE, "squared diagonal exceeds 32 bits");
    if (W * H * L > ws->max_voxels) return fail(RSF_ERR_WORKSPACE_TOO_SMALL, "volume larger than the workspace");
    cudaError_t e = rsf::launch_signed_distance(seed, dtype == RSF_F32, threshold, phi, (int)W, (int)H, (int)L,
                                                reinterpret_cast<unsigned *>(ws->pool_x), (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "signed distance launch");
    return RSF_OK;
}

// The derivative of one step for a batch; kernels and the chain rule are in
// rsf_adjoint.cu.
rsf_status rsf_step_adjoint_batched(rsf_workspace *ws, const rsf_params *p, rsf_dtype dtype,
                                    const rsf_adjoint_subvol *subvols, int32_t n, double *param_grads,
                                    void *stream) {
    if (!ws) return fail(RSF_ERR_INVALID_ARGUMENT, "workspace is null");
    if (!subvols) return fail(RSF_ERR_INVALID_ARGUMENT, "sub-volume array is null");
    if (n < 1) return fail(RSF_ERR_INVALID_ARGUMENT, "batch is empty");
    if (n > ws->max_subvols) return fail(RSF_ERR_WORKSPACE_TOO_SMALL, "more sub-volumes than the workspace holds");
    float taps[rsf::MAXK];
    int k = 0;
    rsf_status s = check_params(p, &k, taps);
    if (s != RSF_OK) return s;
    if ((int)p->sigma2 != 0) return fail(RSF_ERR_UNSUPPORTED, "the adjoint of the box e-term (sigma2 >= 1) is not implemented");
    if (p->data_term != RSF_DATA_TERM_REFERENCE)
        return fail(RSF_ERR_UNSUPPORTED, "the adjoint of the Gaussian data term is not implemented");
    if (dtype != RSF_U8 && dtype != RSF_F32) return fail(RSF_ERR_DTYPE, "image dtype must be RSF_U8 or RSF_F32");
    const size_t esz = dtype == RSF_F32 ? 4 : 1;
    int64_t total = 0;
    for (int i = 0; i < n; i++) {
        const rsf_adjoint_subvol &v = subvols[i];
        if ((s = check_shape(v.W, v.H, v.L)) != RSF_OK) return s;
        if (!v.image || !v.phi || !v.phi_bar_in || !v.phi_bar_out) return fail(RSF_ERR_INVALID_ARGUMENT, "null pointer");
        total += v.W * v.H * v.L;
    }
    if (total > ws->max_voxels) return fail(RSF_ERR_WORKSPACE_TOO_SMALL, "batch larger than the workspace");
    // every output must be disjoint from every input and from the other outputs
    auto overlaps = [](const void *a, size_t abytes, const void *b, size_t bbytes) {
        const char *pa = static_cast<const char *>(a), *pb = static_cast<const char *>(b);
        return pa < pb + bbytes && pb < pa + abytes;
    };
    for (int i = 0; i < n; i++) {
        const rsf_adjoint_subvol &o = subvols[i];
        const size_t ob = (size_t)(o.W * o.H * o.L) * sizeof(float);
        for (int j = 0; j < n; j++) {
            const rsf_adjoint_subvol &v = subvols[j];
            const size_t nv = (size_t)(v.W * v.H * v.L);
            if (overlaps(o.phi_bar_out, ob, v.phi, nv * sizeof(float)) ||
                overlaps(o.phi_bar_out, ob, v.phi_bar_in, nv * sizeof(float)) ||
                overlaps(o.phi_bar_out, ob, v.image, nv * esz) ||
                (j != i && overlaps(o.phi_bar_out, ob, v.phi_bar_out, nv * sizeof(float))))
                return fail(RSF_ERR_INVALID_ARGUMENT, "phi_bar_out overlaps an input or another output");
        }
    }
    cudaStream_t st = (cudaStream_t)stream;
    // Specialised tap counts recompute the blurs with the forward step's own
    // streaming x- and y-passes (pair planes in pool_x, pool_y) and the
    // z-pass's adjoint variant, which leaves the data-term adjoint pair and
    // e_out, e_in in each volume's xs slice.
    const int kspec = rsf::kernel_k(k, RSF_ARITH_PORTABLE, false);
    // The adjoint's table: volume i's scratch slices at the running voxel
    // offset (1, 4 and 4 floats per voxel).
    SubVolDev *h_svs_unused = nullptr;
    int *h_pre_unused = nullptr;
    unsigned char *h_maps_unused = nullptr;
    {
        cudaError_t e = ws->next_stage(&h_svs_unused, &h_pre_unused, &h_maps_unused);
        if (e != cudaSuccess) return cuda_fail(e, "table event");
    }
    const int stg = ws->current_stage();
    rsf::AdjVol *h_adj = ws->h_adj + (size_t)stg * ws->max_subvols;
    int *h_pre = ws->h_adj_pre + (size_t)stg * rsf::NADJ * ((size_t)ws->max_subvols + 1);
    const int n1 = n + 1;
    for (int j = 0; j < rsf::NADJ; j++) h_pre[j * n1] = 0;
    size_t off = 0;
    for (int i = 0; i < n; i++) {
        const rsf_adjoint_subvol &v = subvols[i];
        rsf::AdjVol a;
        a.phi = v.phi;
        a.img = v.image;
        a.u = v.phi_bar_in;
        a.out = v.phi_bar_out;
        a.phi2 = ws->pool_phi2 + off;
        a.xs = ws->pool_x + 4 * off;
        a.ys = ws->pool_y + 4 * off;
        a.W = (int)v.W;
        a.H = (int)v.H;
        a.L = (int)v.L;
        int wp = 0;
        rsf::valid_extents(a.W, a.H, a.L, k, a.Wv, a.Hv, a.Lv, wp);
        off += (size_t)(v.W * v.H * v.L);
        int tiles[rsf::NADJ];
        rsf::adjoint_tiles(a, kspec > 0, tiles);
        for (int j = 0; j < rsf::NADJ; j++) {
            const int64_t next = (int64_t)h_pre[j * n1 + i] + tiles[j];
            if (tiles[j] < 0 || next > 0x7fffffffLL) return fail(RSF_ERR_SHAPE, "batch needs more than 2^31 blocks");
            h_pre[j * n1 + i + 1] = (int)next;
        }
        h_adj[i] = a;
    }
    int tot[rsf::NADJ];
    for (int j = 0; j < rsf::NADJ; j++) tot[j] = h_pre[j * n1 + n];
    cudaError_t e = cudaMemcpyAsync(ws->d_adj, h_adj, (size_t)n * sizeof(rsf::AdjVol), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ws->d_adj_pre, h_pre, rsf::NADJ * (size_t)n1 * sizeof(int), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = ws->mark_stage(st);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint table upload");
    if (kspec > 0) {
        std::vector<rsf_subvol> fw((size_t)n);
        for (int i = 0; i < n; i++)
            fw[i] = rsf_subvol{const_cast<float *>(subvols[i].phi), subvols[i].image, subvols[i].W, subvols[i].H,
                               subvols[i].L};
        int ftot[rsf::NPRE];
        rsf::LaunchShape sh;
        const int saved_zt = ws->force_zt;
        ws->force_zt = 0;  // the adjoint variant streams its planes without TMA
        s = prepare(ws, fw.data(), n, k, kspec, 0, 0, dtype, nullptr, ftot, &sh, st);
        ws->force_zt = saved_zt;
        if (s != RSF_OK) return s;
        const StepConst c = make_const(p, k, taps, dtype, n, sh, nullptr);
        const SubVolDev *svs = ws->d_svs;
        const int *pre = ws->d_pre;
        const int f1 = n + 1;
        if (ftot[0] > 0) switch (kspec) {
                case 21: e = rsf::launch_xpass_21(svs, pre, ftot[0], c, 0, RSF_ARITH_PORTABLE, st); break;
                case 29: e = rsf::launch_xpass_29(svs, pre, ftot[0], c, 0, RSF_ARITH_PORTABLE, st); break;
                default: e = rsf::launch_xpass_35(svs, pre, ftot[0], c, 0, RSF_ARITH_PORTABLE, st); break;
            }
        if (e == cudaSuccess && ftot[1] > 0) switch (kspec) {
                case 21: e = rsf::launch_ypass_21(svs, pre + f1, ftot[1], c, st); break;
                case 29: e = rsf::launch_ypass_29(svs, pre + f1, ftot[1], c, st); break;
                default: e = rsf::launch_ypass_35(svs, pre + f1, ftot[1], c, st); break;
            }
        if (e == cudaSuccess && ftot[2] > 0) switch (kspec) {
                case 21: e = rsf::launch_zpass_adjoint_21(svs, pre + 2 * f1, ftot[2], c, ws->d_adj, st); break;
                case 29: e = rsf::launch_zpass_adjoint_29(svs, pre + 2 * f1, ftot[2], c, ws->d_adj, st); break;
                default: e = rsf::launch_zpass_adjoint_35(svs, pre + 2 * f1, ftot[2], c, ws->d_adj, st); break;
            }
        if (e != cudaSuccess) return cuda_fail(e, "adjoint blur recompute launch");
    }
    const rsf::AdjScalars sc = {p->eps, p->dt, p->mu, p->nu, p->lambda1, p->lambda2, p->boundary, dtype == RSF_F32};
    e = rsf::launch_step_adjoint(taps, k, sc, ws->d_adj, ws->d_adj_pre, n, tot, param_grads, ws->d_flag, st);
    if (e != cudaSuccess) return cuda_fail(e, "adjoint launch");
    return RSF_OK;
}

rsf_status rsf_step_adjoint(rsf_workspace *ws, const rsf_params *p, const void *image, rsf_dtype dtype,
                            const float *phi, const float *phi_bar_in, float *phi_bar_out, double *param_grads,
                            int64_t W, int64_t H, int64_t L, void *stream) {
    const rsf_adjoint_subvol v = {phi, image, phi_bar_in, phi_bar_out, W, H, L};
    return rsf_step_adjoint_batched(ws, p, dtype, &v, 1, param_grads, stream);
}

// Grid checks on the host; the gather itself is in rsf_reassemble.cu.  The
// tile table goes through the workspace's pinned staging and device table.
rsf_status rsf_reassemble(rsf_workspace *ws, const rsf_tile *tiles, int32_t nx, int32_t ny, int32_t nz,
                          const int64_t *core_x, const int64_t *core_y, const int64_t *core_z, int32_t mode,
                          float *out, int64_t W, int64_t H, int64_t L, void *stream) {
    static_assert(sizeof(rsf::TileDev) <= sizeof(SubVolDev), "tile table must fit the sub-volume table");
    if (!ws || !tiles || !core_x || !core_y || !core_z || !out) return fail(RSF_ERR_INVALID_ARGUMENT, "null pointer");
    if (mode != RSF_REASSEMBLE_CORE && mode != RSF_REASSEMBLE_BLEND)
        return fail(RSF_ERR_INVALID_ARGUMENT, "unknown reassembly mode");
    const int n[3] = {nx, ny, nz};
    const int64_t ext[3] = {W, H, L};
    const int64_t *core[3] = {core_x, core_y, core_z};
    for (int a = 0; a < 3; a++) {
        if (n[a] < 1 || n[a] > rsf::RA_MAXCELLS) return fail(RSF_ERR_INVALID_ARGUMENT, "1 to 64 cells per axis");
        if (ext[a] < 1 || ext[a] > kMaxExtent) return fail(RSF_ERR_SHAPE, "bad output extent");
        if (core[a][0] != 0 || core[a][n[a]] != ext[a]) return fail(RSF_ERR_INVALID_ARGUMENT, "cores must span the volume");
        for (int j = 0; j < n[a]; j++)
            if (core[a][j] >= core[a][j + 1]) return fail(RSF_ERR_INVALID_ARGUMENT, "core bounds must increase");
    }
    const int64_t ntiles = (int64_t)nx * ny * nz;
    if (ntiles > ws->max_subvols) return fail(RSF_ERR_WORKSPACE_TOO_SMALL, "more tiles than the workspace holds");
    int cb[3][rsf::RA_MAXCELLS + 1], lo[3][rsf::RA_MAXCELLS], hi[3][rsf::RA_MAXCELLS];
    for (int a = 0; a < 3; a++) {
        for (int j = 0; j <= n[a]; j++) cb[a][j] = (int)core[a][j];
        for (int j = 0; j < n[a]; j++) lo[a][j] = hi[a][j] = -1;
    }
    SubVolDev *h_svs = nullptr;
    int *h_pre = nullptr;
    unsigned char *h_maps = nullptr;
    {
        cudaError_t e = ws->next_stage(&h_svs, &h_pre, &h_maps);
        if (e != cudaSuccess) return cuda_fail(e, "table event");
    }
    rsf::TileDev *h = reinterpret_cast<rsf::TileDev *>(h_svs);
    for (int iz = 0; iz < nz; iz++)
        for (int iy = 0; iy < ny; iy++)
            for (int ix = 0; ix < nx; ix++) {
                const int64_t t = ((int64_t)iz * ny + iy) * nx + ix;
                const rsf_tile &s = tiles[t];
                const int idx[3] = {ix, iy, iz};
                const int64_t o[3] = {s.x0, s.y0, s.z0}, e[3] = {s.W, s.H, s.L};
                if (!s.phi) return fail(RSF_ERR_INVALID_ARGUMENT, "null tile pointer");
                for (int a = 0; a < 3; a++) {
                    const int j = idx[a];
                    if (e[a] < 1 || o[a] < 0 || o[a] + e[a] > ext[a])
                        return fail(RSF_ERR_SHAPE, "tile extends outside the volume");
                    if (o[a] > core[a][j] || o[a] + e[a] < core[a][j + 1])
                        return fail(RSF_ERR_INVALID_ARGUMENT, "tile does not contain its core");
                    if (lo[a][j] < 0) {
                        lo[a][j] = (int)o[a];
                        hi[a][j] = (int)(o[a] + e[a]);
                    } else if (lo[a][j] != (int)o[a] || hi[a][j] != (int)(o[a] + e[a])) {
                        return fail(RSF_ERR_INVALID_ARGUMENT, "tiles of one grid row must share their extent");
                    }
                }
                h[t] = rsf::TileDev{s.phi, (int)s.x0, (int)s.y0, (int)s.z0, (int)s.W, (int)s.H, (int)s.L};
            }
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(ws->d_svs, h, (size_t)ntiles * sizeof(rsf::TileDev), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = ws->mark_stage(st);
    if (e != cudaSuccess) return cuda_fail(e, "tile table upload");
    const int *pcb[3] = {cb[0], cb[1], cb[2]}, *plo[3] = {lo[0], lo[1], lo[2]}, *phi_[3] = {hi[0], hi[1], hi[2]};
    e = rsf::launch_reassemble(reinterpret_cast<const rsf::TileDev *>(ws->d_svs), n, pcb, plo, phi_, mode, out,
                               (int)W, (int)H, (int)L, st);
    if (e != cudaSuccess) return cuda_fail(e, "reassembly launch");
    return RSF_OK;
}

rsf_status rsf_copy_async(void *dst, const void *src, size_t bytes, void *stream) {
    if (bytes == 0) return RSF_OK;
    if (!dst || !src) return fail(RSF_ERR_INVALID_ARGUMENT, "null pointer");
    void *dv = device_view(dst), *sv = device_view(src);
    if (!dv || !sv)
        return fail(RSF_ERR_INVALID_ARGUMENT, "both addresses must be device memory or pinned / registered host memory");
    cudaError_t e = rsf::launch_copy(dv, sv, bytes, (cudaStream_t)stream);
    return e == cudaSuccess ? RSF_OK : cuda_fail(e, "copy launch");
}

rsf_status rsf_workspace_check(rsf_workspace *ws, void *stream) {
    if (!ws) return fail(RSF_ERR_INVALID_ARGUMENT, "workspace is null");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "stream");
    unsigned flag = 0;
    e = cudaMemcpy(&flag, ws->d_flag, sizeof flag, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && flag) e = cudaMemset(ws->d_flag, 0, sizeof flag);
    if (e != cudaSuccess) return cuda_fail(e, "flag read");
    if (flag & rsf::kFlagAdjointNonFinite)
        return fail(RSF_ERR_NONFINITE, "non-finite value in dL/dphi from rsf_step_adjoint (the gradient overflowed FP32)");
    if (flag & rsf::kFlagTimeout) return fail(RSF_ERR_CUDA, "a kernel's barrier wait gave up (TMA copy not completed)");
    if (flag) return fail(RSF_ERR_NONFINITE, "non-finite value written to phi");
    return RSF_OK;
}

rsf_status rsf_set_kernel_timing(rsf_workspace *ws, int enable) {
    if (!ws) return fail(RSF_ERR_INVALID_ARGUMENT, "workspace is null");
    rsf_status s = collect_times(ws);
    if (s != RSF_OK) return s;
    ws->timing = enable != 0;
    return RSF_OK;
}

rsf_status rsf_kernel_times(rsf_workspace *ws, double ms[4], int64_t launches[4], int reset) {
    if (!ws) return fail(RSF_ERR_INVALID_ARGUMENT, "workspace is null");
    rsf_status s = collect_times(ws);
    if (s != RSF_OK) return s;
    for (int j = 0; j < rsf::NKERN; j++) {
        if (ms) ms[j] = ws->kernel_ms[j];
        if (launches) launches[j] = ws->kernel_launches[j];
        if (reset) {
            ws->kernel_ms[j] = 0.0;
            ws->kernel_launches[j] = 0;
        }
    }
    return RSF_OK;
}

}  // extern "C"
