/*
 * rsf.h -- C ABI of the GB300 RSF level-set library (librsf_gb300.so).
 *
 * Region-scalable-fitting level-set evolution of 3-D sub-volumes, as run by
 * the `rsf3d` executable of STIM-Lab/paper-rsf-vesselseg (CUDA_RSF/main.cpp
 * and CUDA_RSF/kernel.cu).  Plain C: pointers, sizes and status codes only.
 *
 * Conventions
 *   - Volumes are dense, x fastest: element (x, y, z) of a W x H x L volume is
 *     at z*W*H + y*W + x (the reference's indexing, CUDA_RSF/kernel.cu:73).
 *     A NumPy array of shape (L, H, W) in C order has this layout.
 *   - Unless a function says "host", pointers are DEVICE pointers owned by
 *     the caller.  Nothing is allocated per call: scratch lives in an
 *     rsf_workspace that the caller creates and destroys explicitly.
 *   - Every call is asynchronous on the given stream (0 = legacy default
 *     stream) and returns an rsf_status; nothing prints, nothing exits.
 *     Errors found while kernels run are reported by rsf_workspace_check().
 *   - A workspace may be used by one stream at a time; different workspaces
 *     are independent and may run concurrently.
 */
#ifndef RSF_GB300_H
#define RSF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RSF_ABI_VERSION 1

typedef enum {
    RSF_OK = 0,
    RSF_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad count, bad parameter */
    RSF_ERR_SHAPE = 2,            /* extent < 2 or too large */
    RSF_ERR_DTYPE = 3,            /* unknown rsf_dtype */
    RSF_ERR_UNSUPPORTED = 4,      /* valid but not implemented combination */
    RSF_ERR_NO_MEMORY = 5,        /* workspace allocation failed */
    RSF_ERR_WORKSPACE_TOO_SMALL = 6,
    RSF_ERR_CUDA = 7,             /* a CUDA runtime call failed */
    RSF_ERR_NONFINITE = 8,        /* NaN/Inf appeared in phi (checked on demand) */
    RSF_ERR_IO = 9,               /* .npy read/write (host helpers) */
    RSF_ERR_NO_DEVICE = 10
} rsf_status;

typedef enum {
    RSF_U8 = 0,  /* uint8 image (the 8-bit stacks the pipeline produces) */
    RSF_F32 = 1  /* float32 image (what the reference loads, main.cpp:148) */
} rsf_dtype;

typedef enum {
    /* x = 0 reads the previous linear element, as the reference's
     * gradient_dx_cuda does (kernel.cu:64-67, an unsigned "j - 1 < 0" test that
     * never fires); voxel 0 reads itself instead of element -1. */
    RSF_BOUNDARY_REFERENCE = 0,
    /* x = 0 uses the one-sided difference (f[1]-f[0])/2 like the y and z rules */
    RSF_BOUNDARY_CLAMP = 1
} rsf_boundary;

typedef enum {
    /* float-only IEEE sequences (compensated where the reference used double,
     * own atan); bit-identical to the CPU oracle on every platform. */
    RSF_ARITH_PORTABLE = 0,
    /* the reference's own arithmetic: CUDA atanf and double precision at the
     * spots kernel.cu evaluates in double.  Slow on GB300 (FP64). */
    RSF_ARITH_REFERENCE = 1
} rsf_arith;

typedef enum {
    /* the reference's data term (kernel.cu:25-55): e = (I - f)^2 at the voxel,
     * or its box sum with sigma2 >= 1 */
    RSF_DATA_TERM_REFERENCE = 0,
    /* the region-scalable fitting energy's data term written out, with no
     * counterpart in the reference: e = I^2 K*1 - 2 I K*f + K*f^2 on the valid
     * region of the blur (K the same valid Gaussian correlation as the fits,
     * f the fit field, 1 in the border band); the border band keeps
     * (I - 1)^2.  Run-time-k kernels; needs sigma2 < 1; no adjoint.  On
     * first use the workspace allocates 16 more bytes per voxel of its
     * capacity for the blurred fields. */
    RSF_DATA_TERM_GAUSSIAN = 1
} rsf_data_term;

/* Parameters of one evolution.  Defaults (rsf_params_default) are the
 * reference's command-line defaults, main.cpp:91-97. */
typedef struct {
    float sigma;    /* --sigma 5.0: Gaussian sigma of the local fit */
    float dt;       /* --dt 0.1 */
    float mu;       /* --meu 1.0: distance-regularisation weight */
    float lambda1;  /* --e 0.1: weight of e_out (inside the phi > 0 region) */
    float lambda2;  /* --e 0.1: weight of e_in */
    float nu;       /* --v 1e-4: curvature (length) weight */
    float eps;      /* 0.2: Heaviside/Dirac width, hard-coded in kernel.cu:258,275 */
    float sigma2;   /* --sigma2 0.0: (int) radius of the e-term box window, 0..8 */
    int32_t boundary; /* rsf_boundary */
    int32_t arith;    /* rsf_arith */
    int32_t data_term; /* rsf_data_term */
    int32_t reserved[5];
} rsf_params;

/* One sub-volume of a batch.  All pointers are device pointers. */
typedef struct {
    float *phi;        /* in/out level set, W*H*L float32 */
    const void *image; /* W*H*L image of the batch's dtype */
    int64_t W, H, L;
} rsf_subvol;

/* One evolved sub-volume placed in a larger volume (rsf_reassemble). */
typedef struct {
    const float *phi;     /* W*H*L float32, device */
    int64_t x0, y0, z0;   /* position of its first voxel in the output */
    int64_t W, H, L;
} rsf_tile;

/* Stitching modes of rsf_reassemble. */
typedef enum {
    RSF_REASSEMBLE_CORE = 0,  /* each voxel from the sub-volume whose core holds it */
    RSF_REASSEMBLE_BLEND = 1  /* linear blend across overlaps */
} rsf_reassemble_mode;

typedef struct rsf_workspace rsf_workspace;

/* Library identification. */
int rsf_abi_version(void);
const char *rsf_status_string(rsf_status s);
/* Message of the last failure on the calling thread (empty if none). */
const char *rsf_last_error(void);

/* Fills the reference defaults. */
rsf_status rsf_params_default(rsf_params *p);

/* The Gaussian taps the evolution uses for `sigma` (main.cpp:152-166:
 * k = floor(7 sigma) made odd, g[i] = exp(-(i-k/2)^2/u)/sqrt(u pi) with
 * u = (int)(2 sigma^2), not normalised).  Host memory; `cap` entries. */
rsf_status rsf_gaussian_taps(float sigma, float *taps_host, int cap, int *k_out);

/* Workspace sized for batches of up to `max_voxels` voxels in total (summed
 * over sub-volumes) and up to `max_subvols` sub-volumes.  Allocates device
 * memory on the current device. */
rsf_status rsf_workspace_create(int64_t max_voxels, int32_t max_subvols, rsf_workspace **ws);
rsf_status rsf_workspace_destroy(rsf_workspace *ws);
/* Bytes of device memory the workspace holds. */
size_t rsf_workspace_bytes(const rsf_workspace *ws);
/* Device bytes a workspace for `max_voxels` / `max_subvols` would hold. */
size_t rsf_workspace_bytes_for(int64_t max_voxels, int32_t max_subvols);

/* Kernel launch shapes for the workspace's later calls, overriding the
 * per-batch heuristics (0, or -1 for z_tma, restores them): x-pass outputs
 * per lane (5 or 9), stencil planes per block (32, 64 or 128) and whether the
 * 21/35-tap z-pass takes its planes through TMA (1) or the streaming ring
 * (0).  Results do not depend on the choice (every shape is bit-identical);
 * rsf_gb300.autotune.tune_launch_shape measures them on a batch.  No
 * counterpart in the reference, whose launch shapes are fixed in kernel.cu. */
rsf_status rsf_workspace_set_launch_shape(rsf_workspace *ws, int32_t xpass_width, int32_t stencil_planes,
                                          int32_t z_tma);

/* Evolves one volume in place for `iters` iterations: the device-resident
 * equivalent of the reference's hot loop (main.cpp:222-314).
 * Replaces the per-op host wrappers declared at main.cpp:56-71. */
rsf_status rsf_evolve(rsf_workspace *ws, const rsf_params *p, const void *image, rsf_dtype dtype,
                      float *phi, int64_t W, int64_t H, int64_t L, int32_t iters, void *stream);

/* Evolves `n` independent sub-volumes of (possibly) different shapes in one
 * launch sequence per iteration, the iteration loop captured once into a
 * CUDA graph and replayed.  Replaces the one-process-per-sub-volume batch
 * driver described at README.md:56 (rsfbatch.py, not in the reference). */
rsf_status rsf_evolve_batched(rsf_workspace *ws, const rsf_params *p, rsf_dtype dtype,
                              const rsf_subvol *subvols, int32_t n, int32_t iters, void *stream);

/* Host-buffer convenience: copies image and phi to the device, evolves,
 * copies phi back (synchronous).  `phi_host` is updated in place.  This is
 * the call shape of the reference's wrappers (host pointers in and out). */
rsf_status rsf_evolve_host(rsf_workspace *ws, const rsf_params *p, const void *image_host,
                           rsf_dtype dtype, float *phi_host, int64_t W, int64_t H, int64_t L,
                           int32_t iters);

/* One iteration with the intermediate fields written out, for parity
 * checks.  `fields` receives 8 W*H*L float32 volumes in this order:
 * f_out, f_in, e_out, e_in, delta, kappa, laplacian, |grad phi|
 * (the reference's fout_x, fin_x, Eout, Ein, derivative_heaviside,
 * normalized_DIV, DIV, Gradientmagnitude_phi; main.cpp:195-211).
 * phi_out receives the updated level set; phi is not modified. */
rsf_status rsf_step_debug(rsf_workspace *ws, const rsf_params *p, const void *image,
                          rsf_dtype dtype, const float *phi, float *phi_out, float *fields,
                          int64_t W, int64_t H, int64_t L, void *stream);

/* Per-kernel device timing.  When enabled, every evolution records CUDA
 * events before and after each of its four kernels (x-pass, y-pass, z-pass,
 * stencil/update), inside captured graphs too; rsf_kernel_times waits for
 * them and returns the accumulated milliseconds and launch counts. */
rsf_status rsf_set_kernel_timing(rsf_workspace *ws, int enable);
rsf_status rsf_kernel_times(rsf_workspace *ws, double ms[4], int64_t launches[4], int reset);

/* Evolution without any device allocation, for callers that cannot
 * allocate once running: plug-ins inside an application that owns the
 * device memory budget through its own pool, real-time loops that forbid
 * allocation after start-up.  Same arguments and result as rsf_evolve, but
 * no workspace: all scratch lives in one static device array of this
 * library (about 36 MiB), reserved when its module loads on a device and
 * held until the process exits.  Limit: W*H*L <= 1048576 voxels; larger
 * volumes return RSF_ERR_WORKSPACE_TOO_SMALL.  The first call on a device
 * looks up the array's device address and configures the kernels; make it
 * before any stream capture (a first call on a capturing stream returns
 * RSF_ERR_UNSUPPORTED).  The address is cached for the process: calls after
 * cudaDeviceReset on that device are not supported.
 * Every call shares the array and finds the previous call's contents in it;
 * calls whose work overlaps on one GPU (for instance on two streams) race on
 * the array and corrupt each other: serialise them.  Non-finite values are
 * not reported.
 * This entry point has no counterpart in the reference. */
rsf_status rsf_evolve_noalloc(const rsf_params *p, const void *image, rsf_dtype dtype, float *phi,
                              int64_t W, int64_t H, int64_t L, int32_t iters, void *stream);

/* Initial level set from a seed volume (replaces CUDA_RSF/main.cpp:174-183,
 * which subtracts 13 from the seed and calls tiralib's volume::sdf()).
 * A voxel is inside when seed > threshold (13 in the reference).  phi
 * receives the exact signed Euclidean distance in voxels between voxel
 * centres: +distance to the nearest outside voxel at inside voxels,
 * -distance to the nearest inside voxel at outside voxels.  When one class
 * is empty the other is filled with +-(W + H + L).  seed is a device volume
 * of RSF_U8 or RSF_F32, phi a device float volume of the same shape.
 * Scratch comes from the workspace (ws must hold >= W*H*L voxels); needs
 * (W-1)^2 + (H-1)^2 + (L-1)^2 < 2^32 - 1. */
rsf_status rsf_signed_distance(rsf_workspace *ws, const void *seed, rsf_dtype dtype, float threshold, float *phi,
                               int64_t W, int64_t H, int64_t L, void *stream);

/* Reverse-mode derivative of one evolution step phi -> phi' (the step of
 * CUDA_RSF/main.cpp:233-300; no counterpart in the reference, which has no
 * derivative).  Given phi (the state before the step) and phi_bar_in =
 * dL/dphi', writes phi_bar_out = dL/dphi and, when param_grads is not NULL,
 * ADDS dL/dlambda1, dL/dlambda2, dL/dmu, dL/dnu to param_grads[0..3] (device
 * doubles), so a chain of calls sums them over the steps.  The data term is
 * differentiated as lambda1 e_out - lambda2 e_in with both weights
 * independent (for tied weights add the two).  The derivative is that of the
 * real-valued step evaluated in FP32 (p->arith is ignored); the box e-term
 * (sigma2 >= 1) has no adjoint here (RSF_ERR_UNSUPPORTED).  phi_bar_out must not overlap phi,
 * phi_bar_in or the image.  Scratch comes from the workspace (ws must hold
 * >= W*H*L voxels); parameter sums use atomics, so their last bits may vary
 * from run to run. */
rsf_status rsf_step_adjoint(rsf_workspace *ws, const rsf_params *p, const void *image, rsf_dtype dtype,
                            const float *phi, const float *phi_bar_in, float *phi_bar_out, double *param_grads,
                            int64_t W, int64_t H, int64_t L, void *stream);

/* One volume of an adjoint batch (rsf_step_adjoint_batched): the arguments
 * of rsf_step_adjoint for that volume. */
typedef struct {
    const float *phi;        /* state before the step, W*H*L float32, device */
    const void *image;       /* W*H*L image of the batch's dtype */
    const float *phi_bar_in; /* dL/dphi' */
    float *phi_bar_out;      /* dL/dphi (written) */
    int64_t W, H, L;
} rsf_adjoint_subvol;

/* rsf_step_adjoint for n volumes that share the step parameters, as one
 * launch sequence over the batch (the table of rsf_evolve_batched's kind).
 * param_grads (device doubles, may be NULL) receives the parameter
 * gradients summed over the batch.  Each phi_bar_out must be disjoint from
 * every input and from the other outputs.  The workspace must hold the
 * batch's total voxels and n sub-volumes. */
rsf_status rsf_step_adjoint_batched(rsf_workspace *ws, const rsf_params *p, rsf_dtype dtype,
                                    const rsf_adjoint_subvol *subvols, int32_t n, double *param_grads,
                                    void *stream);

/* Stitches a grid of evolved sub-volumes into `out` (W*H*L float32, device),
 * the step of the reference's missing reassemble.py (README.md:9) and of
 * interpolating_volumes.py:10-40.  Core boundaries core_x[0..nx] (0 .. W),
 * core_y[0..ny], core_z[0..nz] partition the volume; tiles[(iz*ny + iy)*nx +
 * ix] holds cell (ix, iy, iz), must contain its core box and must share its
 * x extent with every tile of index ix (likewise y, z).  RSF_REASSEMBLE_CORE
 * copies each core; RSF_REASSEMBLE_BLEND weights each tile, per axis, by a
 * ramp rising from 0 to 1 in equal steps across its overlap with the
 * previous tile and falling across its overlap with the next (the weights of
 * interpolating_volumes.py), multiplies the axes and normalises.  At most
 * 64 cells per axis and max_subvols tiles; the tile table travels through
 * the workspace. */
rsf_status rsf_reassemble(rsf_workspace *ws, const rsf_tile *tiles, int32_t nx, int32_t ny, int32_t nz,
                          const int64_t *core_x, const int64_t *core_y, const int64_t *core_z, int32_t mode,
                          float *out, int64_t W, int64_t H, int64_t L, void *stream);

/* Copies `bytes` from src to dst with the device's SMs (16-byte loads and
 * stores), asynchronously on `stream`.  Both addresses must be accessible
 * from the device: device memory, or host memory that is pinned
 * (cudaHostAlloc / cudaMallocHost) or registered (cudaHostRegister);
 * RSF_ERR_INVALID_ARGUMENT otherwise (pageable host memory).  On GB300 it
 * keeps about 210 GB/s between pinned host memory and the device where the
 * copy engine's rate falls to 53-69 GB/s once kernels have run; the
 * host-buffer entry points use it.  No counterpart in the reference. */
rsf_status rsf_copy_async(void *dst, const void *src, size_t bytes, void *stream);

/* Waits for the workspace's stream work and reports kernel-side errors
 * (non-finite phi when checking is enabled, CUDA launch errors). */
rsf_status rsf_workspace_check(rsf_workspace *ws, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RSF_GB300_H */
