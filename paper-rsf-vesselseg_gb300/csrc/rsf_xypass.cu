// rsf_xypass.cu -- fused x/y-pass for one tap count (compiled once per
// -DRSF_K value, 21 or 35).
#include "rsf_xy.cuh"
#include "rsf_zt.cuh"

#ifndef RSF_K
#error "compile with -DRSF_K=<taps>"
#endif
#define RSF_CAT2(a, b) a##b
#define RSF_CAT(a, b) RSF_CAT2(a, b)

namespace rsf {

cudaError_t RSF_CAT(config_xypass_, RSF_K)() {
    return cudaFuncSetAttribute(xypass_kernel<RSF_K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)xy_smem_bytes(XY_TX_MAX, RSF_K));
}

cudaError_t RSF_CAT(launch_xypass_, RSF_K)(const SubVolDev *svs, const int *pre, int blocks, const StepConst &c,
                                           int parity, cudaStream_t st) {
    if (c.xy_tx < XY_TX_MIN || c.xy_tx > XY_TX_MAX || c.xy_tx % XY_R != 0) return cudaErrorInvalidValue;
    xypass_kernel<RSF_K><<<blocks, 2 * c.xy_tx, xy_smem_bytes(c.xy_tx, RSF_K), st>>>(svs, pre, c, parity);
    return cudaGetLastError();
}

cudaError_t RSF_CAT(launch_ztpass_, RSF_K)(const SubVolDev *svs, const int *pre, int blocks, const StepConst &c,
                                           unsigned *flag, cudaStream_t st) {
    if (!c.ymaps) return cudaErrorInvalidValue;
    ztpass_kernel<RSF_K><<<blocks, ZT_THREADS, 0, st>>>(svs, pre, c, flag);
    return cudaGetLastError();
}

}  // namespace rsf
