// rsf_zpass.cu -- z-pass (local fits and data factor) for one tap count
// (compiled once per -DRSF_K value; RSF_K = 0 is the run-time-k kernel, which
// also writes the debug fields).  The specialised tap counts also carry the
// adjoint's variant, which emits the data-term adjoint instead of the data
// factor.
#include "rsf_kernels.cuh"

#ifndef RSF_K
#error "compile with -DRSF_K=<taps>"
#endif
#define RSF_CAT2(a, b) a##b
#define RSF_CAT(a, b) RSF_CAT2(a, b)

namespace rsf {

cudaError_t RSF_CAT(launch_zpass_, RSF_K)(const SubVolDev *svs, const int *pre, int blocks, const StepConst &c,
                                          const DebugOut *dbg, cudaStream_t st) {
    const DebugOut none = {nullptr, 0};
#if RSF_K > 0
    (void)dbg;
#if RSF_K == 35
    if (c.pairs) zpass_wide_kernel<RSF_K, true><<<blocks, ZP_PAIRS * 4, 0, st>>>(svs, pre, c);
#else
    if (c.pairs) zpass_kernel<RSF_K, false, true><<<blocks, ZP_PAIRS * 4, 0, st>>>(svs, pre, c, none);
#endif
    else zpass_kernel<RSF_K, false, false><<<blocks, ZP_PAIRS * 4, 0, st>>>(svs, pre, c, none);
#else
    if (dbg) zpass_generic_kernel<true><<<blocks, ZB_TX, 0, st>>>(svs, pre, c, *dbg);
    else zpass_generic_kernel<false><<<blocks, ZB_TX, 0, st>>>(svs, pre, c, none);
#endif
    return cudaGetLastError();
}

#if RSF_K > 0
cudaError_t RSF_CAT(launch_zpass_adjoint_, RSF_K)(const SubVolDev *svs, const int *pre, int blocks,
                                                  const StepConst &c, const AdjVol *vols, cudaStream_t st) {
    zpass_adjoint_kernel<RSF_K><<<blocks, ZP_PAIRS * 4, 0, st>>>(svs, pre, c, vols);
    return cudaGetLastError();
}
#endif

}  // namespace rsf
