// rsf_arith.cuh -- pointwise arithmetic of the RSF step on the device.
//
// Every operation is an explicit correctly-rounded intrinsic (__fmaf_rn,
// __fmul_rn, __fadd_rn, __fsub_rn, __fdiv_rn, __frcp_rn, __fsqrt_rn), so nvcc can neither
// contract nor reorder anything.  The portable definitions (Arith::Portable)
// are the exact same operation sequences as the CPU oracle's, which makes the
// GPU result bit-identical to the oracle on every input.  Arith::Reference
// reproduces the reference kernels' own evaluation (CUDA atanf and double
// precision at the spots CUDA_RSF/kernel.cu evaluates in double).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rsf {

enum class Arith : int { Portable = 0, Reference = 1 };

// atan(u) = u + u^3 R(u^2) on [0, 1] with R fitted for this project (degree
// 8, weighted least squares towards minimax relative error; max error 0.95
// ulp on [-1, 1], 1.35 ulp beyond),
// and atan(x) = pi/2 - atan(1/x) above 1.
__device__ __forceinline__ float atan_portable(float x) {
    const float a = fabsf(x);
    const bool big = a > 1.0f;
    const float u = big ? __frcp_rn(a) : a;  // the correctly rounded 1/a, as 1.0f / a
    const float z = __fmul_rn(u, u);
    float r = -0x1.d727360000000p-10f;
    r = __fmaf_rn(r, z, 0x1.6636cc0000000p-7f);
    r = __fmaf_rn(r, z, -0x1.ff5ed60000000p-6f);
    r = __fmaf_rn(r, z, 0x1.db15280000000p-5f);
    r = __fmaf_rn(r, z, -0x1.584c200000000p-4f);
    r = __fmaf_rn(r, z, 0x1.c0a2c00000000p-4f);
    r = __fmaf_rn(r, z, -0x1.2422a20000000p-3f);
    r = __fmaf_rn(r, z, 0x1.9992160000000p-3f);
    r = __fmaf_rn(r, z, -0x1.55553e0000000p-2f);
    const float t = __fmul_rn(u, z);
    const float p = __fmaf_rn(t, r, u);
    const float res = big ? __fadd_rn(__fsub_rn(0x1.921fb60000000p+0f, p), -0x1.777a5c0000000p-25f) : p;
    return copysignf(res, x);
}

// H = 0.5 (1 + (2/pi) atan(phi/eps)), CUDA_RSF/kernel.cu:258-259.  With
// eps = 1 (a launch-wide value) phi / eps is phi itself, exactly.
template <Arith A>
__device__ __forceinline__ float heaviside(float phi, float eps) {
    float q;
    if (eps == 1.0f) q = phi;
    else q = __fdiv_rn(phi, eps);
    if constexpr (A == Arith::Reference) {
        const float a = atanf(q);
        const double v = __dmul_rn(0.5, __fma_rn(2.0 / 3.14159265358979323846, (double)a, 1.0));
        return __double2float_rn(v);
    } else {
        const float a = atan_portable(q);
        const float TWO_PI_HI = 0x1.45f3060000000p-1f, TWO_PI_LO = 0x1.b939100000000p-26f;
        const float p = __fmul_rn(TWO_PI_HI, a);
        const float pe = __fmaf_rn(TWO_PI_HI, a, -p);
        const float s = __fadd_rn(1.0f, p);
        const float se = __fadd_rn(__fsub_rn(1.0f, s), p);
        const float lo = __fadd_rn(__fmaf_rn(TWO_PI_LO, a, pe), se);
        return __fmul_rn(0.5f, __fadd_rn(s, lo));
    }
}

// delta = (1/pi) eps / (eps^2 + phi^2), CUDA_RSF/kernel.cu:275-276.  (For
// eps = 1 the quotient equals __frcp_rn of the denominator, but the stencil
// measured slower with that branch: 11.5 against 10.1 ms per launch.)
template <Arith A>
__device__ __forceinline__ float dirac(float phi, float eps) {
    const float q = __fdiv_rn(eps, __fmaf_rn(phi, phi, __fmul_rn(eps, eps)));
    if constexpr (A == Arith::Reference) {
        return __double2float_rn(__dmul_rn(1.0 / 3.14159265358979323846, (double)q));
    } else {
        const float INV_PI_HI = 0x1.45f3060000000p-2f, INV_PI_LO = 0x1.b939100000000p-27f;
        const float p = __fmul_rn(INV_PI_HI, q);
        const float e = __fmaf_rn(INV_PI_HI, q, -p);
        return __fadd_rn(p, __fmaf_rn(INV_PI_LO, q, e));
    }
}

// Central difference (r - l)/2; equal to the reference's double evaluation
// (kernel.cu:73-76) because the difference of two floats is exact in double
// and halving commutes with rounding.
__device__ __forceinline__ float half_diff(float r, float l) { return __fmul_rn(__fsub_rn(r, l), 0.5f); }

// |g| = sqrt(gx*gx + gy*gy + gz*gz) with nvcc's contraction of kernel.cu:928.
__device__ __forceinline__ float grad_mag(float gx, float gy, float gz) {
    return __fsqrt_rn(__fmaf_rn(gz, gz, __fmaf_rn(gx, gx, __fmul_rn(gy, gy))));
}

// n_a = g_a / (|g| + 1e-6), kernel.cu:185 (double in the reference).
struct NormDen {
    float s, dlo, rinv;
    double dref;
};

template <Arith A>
__device__ __forceinline__ NormDen norm_den(float mag) {
    NormDen d;
    if constexpr (A == Arith::Reference) {
        d.dref = __dadd_rn((double)mag, 1e-6);
        d.s = d.dlo = d.rinv = 0.0f;
    } else {
        const float EPS6_HI = 0x1.0c6f7a0000000p-20f, EPS6_LO = 0x1.6bdb1a0000000p-49f;
        d.s = __fadd_rn(mag, EPS6_HI);
        const float bb = __fsub_rn(d.s, mag);
        const float err = __fadd_rn(__fsub_rn(mag, __fsub_rn(d.s, bb)), __fsub_rn(EPS6_HI, bb));
        d.dlo = __fadd_rn(err, EPS6_LO);
        d.rinv = __frcp_rn(d.s);  // the correctly rounded 1 / s, as 1.0f / s
        d.dref = 0.0;
    }
    return d;
}

template <Arith A>
__device__ __forceinline__ float normalise(float g, const NormDen &d) {
    if constexpr (A == Arith::Reference) {
        return __double2float_rn(__ddiv_rn((double)g, d.dref));
    } else {
        const float q0 = __fmul_rn(g, d.rinv);
        float r = __fmaf_rn(-q0, d.s, g);
        r = __fmaf_rn(-q0, d.dlo, r);
        return __fmaf_rn(r, d.rinv, q0);
    }
}

// Final_phi, kernel.cu:384, with nvcc's contraction:
//   fma(mu, dt*(lap-kap), fma((nu*dt)*dh, kap, fma(-(dh*data), dt, phi)))
__device__ __forceinline__ float update_phi(float phi, float dh, float data, float kap, float lap,
                                            float dt, float nu, float mu) {
    const float a = __fmaf_rn(-__fmul_rn(dh, data), dt, phi);
    const float b = __fmaf_rn(__fmul_rn(__fmul_rn(nu, dt), dh), kap, a);
    return __fmaf_rn(mu, __fmul_rn(dt, __fsub_rn(lap, kap)), b);
}

// lambda (e_out - e_in) when lambda1 == lambda2 (the reference's single --e),
// else lambda1 e_out - lambda2 e_in.
__device__ __forceinline__ float data_factor(float eo, float ei, float l1, float l2, bool equal) {
    return equal ? __fmul_rn(l1, __fsub_rn(eo, ei)) : __fsub_rn(__fmul_rn(l1, eo), __fmul_rn(l2, ei));
}

}  // namespace rsf
