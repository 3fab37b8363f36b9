// rsf_ztpass.cu -- the TMA-fed z-pass for one tap count (compiled once per
// -DRSF_K value, 21 or 35).
#include "rsf_zt.cuh"

#ifndef RSF_K
#error "compile with -DRSF_K=<taps>"
#endif
#define RSF_CAT2(a, b) a##b
#define RSF_CAT(a, b) RSF_CAT2(a, b)

namespace rsf {

cudaError_t RSF_CAT(config_ztpass_, RSF_K)() {
    return cudaFuncSetAttribute(ztpass_kernel<RSF_K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)zt_smem_bytes(RSF_K));
}

cudaError_t RSF_CAT(launch_ztpass_, RSF_K)(const SubVolDev *svs, const int *pre, int blocks, const StepConst &c,
                                           unsigned *flag, cudaStream_t st) {
    if (!c.ymaps) return cudaErrorInvalidValue;
    ztpass_kernel<RSF_K><<<blocks, ZT_THREADS, zt_smem_bytes(RSF_K), st>>>(svs, pre, c, flag);
    return cudaGetLastError();
}

}  // namespace rsf
