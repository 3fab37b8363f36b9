// rsf_copy.cu -- copies between device memory and pinned host memory with
// the SMs: a grid of 16-byte loads and stores.
//
// On the GB300 (Grace host over NVLink-C2C) the copy engine's host-to-device
// rate was measured at about 210 GB/s on an idle device but 53-69 GB/s after
// the device had run kernels, while SM loads from pinned host memory kept
// about 210 GB/s; the host-buffer paths therefore pull and push their data
// with this kernel.  Both addresses must be accessible from the device
// (device memory, or host memory that is pinned or registered).
#include <cuda_runtime.h>

#include <cstdint>

#include "rsf_internal.h"

namespace rsf {
namespace {

__global__ void __launch_bounds__(512) copy16_kernel(const uint4 *__restrict__ src, uint4 *__restrict__ dst, size_t n) {
    for (size_t i = (size_t)blockIdx.x * 512 + threadIdx.x; i < n; i += (size_t)gridDim.x * 512) dst[i] = src[i];
}

__global__ void __launch_bounds__(256) copy1_kernel(const unsigned char *__restrict__ src,
                                                    unsigned char *__restrict__ dst, size_t n) {
    for (size_t i = (size_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (size_t)gridDim.x * 256) dst[i] = src[i];
}

}  // namespace

cudaError_t launch_copy(void *dst, const void *src, size_t bytes, cudaStream_t st) {
    if (bytes == 0) return cudaSuccess;
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst), b = reinterpret_cast<uintptr_t>(src);
    size_t head = 0;
    const size_t max_blocks = 8 * (size_t)sm_count();
    if ((a & 15) == 0 && (b & 15) == 0) {
        const size_t n16 = bytes / 16;
        if (n16 > 0) {
            size_t blocks = (n16 + 511) / 512;
            if (blocks > max_blocks) blocks = max_blocks;
            copy16_kernel<<<(unsigned)blocks, 512, 0, st>>>(static_cast<const uint4 *>(src), static_cast<uint4 *>(dst),
                                                            n16);
        }
        head = n16 * 16;
    }
    const size_t rest = bytes - head;
    if (rest > 0) {
        size_t blocks = (rest + 255) / 256;
        if (blocks > max_blocks) blocks = max_blocks;
        copy1_kernel<<<(unsigned)blocks, 256, 0, st>>>(static_cast<const unsigned char *>(src) + head,
                                                       static_cast<unsigned char *>(dst) + head, rest);
    }
    return cudaGetLastError();
}

}  // namespace rsf
