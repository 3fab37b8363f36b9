// rsf_xpass.cu -- x-pass instantiations for one tap count (compiled once per
// -DRSF_K value; RSF_K = 0 is the run-time-k kernel, which also serves the
// reference arithmetic).
#include "rsf_kernels.cuh"

#ifndef RSF_K
#error "compile with -DRSF_K=<taps>"
#endif
#define RSF_CAT2(a, b) a##b
#define RSF_CAT(a, b) RSF_CAT2(a, b)

namespace rsf {

static size_t xpass_smem(int k, int xb) {
    const int span = 32 * xb + k - 1;
    return sizeof(float4) * (size_t)XP_ROWS * span + sizeof(float2) * MAXK + sizeof(float) * XP_ROWS * 2 * 32 * xb;
}

template <int XB, Arith A>
static cudaError_t allow(int k) {
    return cudaFuncSetAttribute(xpass_kernel<RSF_K, XB, A>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)xpass_smem(k, XB));
}

cudaError_t RSF_CAT(config_xpass_, RSF_K)() {
    const int kmax = RSF_K > 0 ? RSF_K : MAXK;
    cudaError_t e = allow<5, Arith::Portable>(kmax);
    if (e == cudaSuccess) e = allow<9, Arith::Portable>(kmax);
#if RSF_K == 0
    if (e == cudaSuccess) e = allow<5, Arith::Reference>(kmax);
    if (e == cudaSuccess) e = allow<9, Arith::Reference>(kmax);
#endif
    return e;
}

cudaError_t RSF_CAT(launch_xpass_, RSF_K)(const SubVolDev *svs, const int *pre, int blocks, const StepConst &c,
                                          int parity, int arith, cudaStream_t st) {
    const size_t smem = xpass_smem(RSF_K > 0 ? RSF_K : c.k, c.xb_w);
    constexpr int T = XP_ROWS * 32;
#if RSF_K == 0
    if (arith == 1) {
        if (c.xb_w == 5) xpass_kernel<0, 5, Arith::Reference><<<blocks, T, smem, st>>>(svs, pre, c, parity);
        else xpass_kernel<0, 9, Arith::Reference><<<blocks, T, smem, st>>>(svs, pre, c, parity);
        return cudaGetLastError();
    }
#else
    (void)arith;
#endif
    if (c.xb_w == 5) xpass_kernel<RSF_K, 5, Arith::Portable><<<blocks, T, smem, st>>>(svs, pre, c, parity);
    else xpass_kernel<RSF_K, 9, Arith::Portable><<<blocks, T, smem, st>>>(svs, pre, c, parity);
    return cudaGetLastError();
}

}  // namespace rsf
