// rsf_ypass.cu -- y-pass for one tap count (compiled once per -DRSF_K value;
// RSF_K = 0 is the run-time-k register-blocked kernel).
#include "rsf_kernels.cuh"

#ifndef RSF_K
#error "compile with -DRSF_K=<taps>"
#endif
#define RSF_CAT2(a, b) a##b
#define RSF_CAT(a, b) RSF_CAT2(a, b)

namespace rsf {

cudaError_t RSF_CAT(launch_ypass_, RSF_K)(const SubVolDev *svs, const int *pre, int blocks, const StepConst &c,
                                          cudaStream_t st) {
#if RSF_K > 0
    ypass_kernel<RSF_K><<<blocks, YP_COLS, 0, st>>>(svs, pre, c);
#else
    ypass_generic_kernel<0><<<blocks, YB_TX, 0, st>>>(svs, pre, c);
#endif
    return cudaGetLastError();
}

}  // namespace rsf
