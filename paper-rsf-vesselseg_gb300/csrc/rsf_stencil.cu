// rsf_stencil.cu -- the stencil / update kernel instantiations.
#include "rsf_kernels.cuh"

namespace rsf {

cudaError_t launch_stencil(const SubVolDev *svs, const int *pre, int blocks, const StepConst &c, int parity,
                           int arith, unsigned *flag, const DebugOut *dbg, cudaStream_t st) {
    const DebugOut none = {nullptr, 0};
    constexpr int T = ST_WARPS * 32;
    if (dbg) {
        if (arith == 1) stencil_kernel<Arith::Reference, true><<<blocks, T, 0, st>>>(svs, pre, c, parity, flag, *dbg);
        else stencil_kernel<Arith::Portable, true><<<blocks, T, 0, st>>>(svs, pre, c, parity, flag, *dbg);
    } else {
        if (arith == 1) stencil_kernel<Arith::Reference, false><<<blocks, T, 0, st>>>(svs, pre, c, parity, flag, none);
        else stencil_kernel<Arith::Portable, false><<<blocks, T, 0, st>>>(svs, pre, c, parity, flag, none);
    }
    return cudaGetLastError();
}

cudaError_t launch_box(const SubVolDev *svs, const int *pre, int blocks, const StepConst &c, const DebugOut *dbg,
                       cudaStream_t st) {
    constexpr int T = ST_WARPS * 32;
    if (dbg) box_kernel<true><<<blocks, T, 0, st>>>(svs, pre, c, *dbg);
    else box_kernel<false><<<blocks, T, 0, st>>>(svs, pre, c, DebugOut{nullptr, 0});
    return cudaGetLastError();
}

}  // namespace rsf
