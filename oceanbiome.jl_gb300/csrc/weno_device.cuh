// weno_device.cuh — upwind-biased WENO reconstructions used by the tracer advection.
//
// Oceananigans' WENO(order = 5) (the scheme the reference's examples pass as `advection`) is a
// third-party routine absent from this tree; it is restated here from the published WENO-Z
// scheme (Borges, Carmona, Costa & Don 2008) with p = 2 and eps = 1e-8, with the order reduced to
// WENO3 and then to first-order upwinding where a Bounded wall leaves fewer than three cells on
// either side of a face.
//
// Each function returns the reconstruction at the face downwind of v3 (WENO5) or v2 (WENO3),
// given values ordered from far upwind to downwind; the caller mirrors the stencil for U < 0.
#pragma once
#include "obgc_common.cuh"

namespace obgc {

template <typename T>
__host__ __device__ __forceinline__ T weno5(T v1, T v2, T v3, T v4, T v5) {
    const T eps = T(1e-8);
    const T c6 = T(1.0 / 6.0);
    const T q0 = (T(2) * v1 - T(7) * v2 + T(11) * v3) * c6;
    const T q1 = (-v2 + T(5) * v3 + T(2) * v4) * c6;
    const T q2 = (T(2) * v3 + T(5) * v4 - v5) * c6;
    T a = v1 - T(2) * v2 + v3, b = v1 - T(4) * v2 + T(3) * v3;
    const T b0 = T(13.0 / 12.0) * a * a + T(0.25) * b * b;
    a = v2 - T(2) * v3 + v4; b = v2 - v4;
    const T b1 = T(13.0 / 12.0) * a * a + T(0.25) * b * b;
    a = v3 - T(2) * v4 + v5; b = T(3) * v3 - T(4) * v4 + v5;
    const T b2 = T(13.0 / 12.0) * a * a + T(0.25) * b * b;
    const T tau = t_abs(b0 - b2);
    const T r0 = tau / (b0 + eps), r1 = tau / (b1 + eps), r2 = tau / (b2 + eps);
    const T a0 = T(0.1) * (T(1) + r0 * r0);
    const T a1 = T(0.6) * (T(1) + r1 * r1);
    const T a2 = T(0.3) * (T(1) + r2 * r2);
    return (a0 * q0 + a1 * q1 + a2 * q2) / (a0 + a1 + a2);
}

// FP32 specialisation.  The same formula in difference form: with d_k = v_k - v3 the candidate
// polynomials are v3 + p_k and the smoothness indicators depend on the d_k only, so they keep full
// relative precision when the stencil holds nearly equal large values (NO3 ~ 10, DIC ~ 2000), where
// the direct form loses the differences to cancellation.  Approximate reciprocals: four MUFU ops per
// face instead of four IEEE divisions (rcp.approx has <= 1 ulp error; its arguments are
// >= 1e-8 (beta + eps) and >= 1 (sum of alphas), so flushing subnormals is moot).
#ifdef __CUDA_ARCH__
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
// The operation sequence matches weno5_x2 (weno_x2.cuh) element for element, so a face rounds the
// same whichever of the two computes it.
template <>
__device__ __forceinline__ float weno5<float>(float v1, float v2, float v3, float v4, float v5) {
    const float eps = 1e-8f;
    const float d1 = __fsub_rn(v1, v3), d2 = __fsub_rn(v2, v3), d4 = __fsub_rn(v4, v3), d5 = __fsub_rn(v5, v3);
    const float p0 = fmaf(2.f / 6.f, d1, __fmul_rn(-7.f / 6.f, d2));
    const float p1 = fmaf(-1.f / 6.f, d2, __fmul_rn(2.f / 6.f, d4));
    const float p2 = fmaf(5.f / 6.f, d4, __fmul_rn(-1.f / 6.f, d5));
    float a = fmaf(-2.f, d2, d1);
    float b = fmaf(-4.f, d2, d1);
    const float b0 = fmaf(__fmul_rn(13.f / 12.f, a), a, __fmul_rn(__fmul_rn(0.25f, b), b));
    a = __fadd_rn(d2, d4);
    b = __fsub_rn(d2, d4);
    const float b1 = fmaf(__fmul_rn(13.f / 12.f, a), a, __fmul_rn(__fmul_rn(0.25f, b), b));
    a = fmaf(-2.f, d4, d5);
    b = fmaf(-4.f, d4, d5);
    const float b2 = fmaf(__fmul_rn(13.f / 12.f, a), a, __fmul_rn(__fmul_rn(0.25f, b), b));
    const float tau = fabsf(__fsub_rn(b0, b2));
    const float r0 = __fmul_rn(tau, rcp_approx(__fadd_rn(b0, eps)));
    const float r1 = __fmul_rn(tau, rcp_approx(__fadd_rn(b1, eps)));
    const float r2 = __fmul_rn(tau, rcp_approx(__fadd_rn(b2, eps)));
    const float a0 = __fmul_rn(0.1f, fmaf(r0, r0, 1.f));
    const float a1 = __fmul_rn(0.6f, fmaf(r1, r1, 1.f));
    const float a2 = __fmul_rn(0.3f, fmaf(r2, r2, 1.f));
    const float num = fmaf(a0, p0, fmaf(a1, p1, __fmul_rn(a2, p2)));
    return fmaf(num, rcp_approx(__fadd_rn(__fadd_rn(a0, a1), a2)), v3);
}
#endif

template <typename T>
__host__ __device__ __forceinline__ T weno3(T v1, T v2, T v3) {
    const T eps = T(1e-8);
    const T q0 = (-v1 + T(3) * v2) * T(0.5), q1 = (v2 + v3) * T(0.5);
    const T b0 = (v2 - v1) * (v2 - v1), b1 = (v3 - v2) * (v3 - v2);
    const T tau = t_abs(b0 - b1);
    const T r0 = tau / (b0 + eps), r1 = tau / (b1 + eps);
    const T a0 = T(1.0 / 3.0) * (T(1) + r0 * r0), a1 = T(2.0 / 3.0) * (T(1) + r1 * r1);
    return (a0 * q0 + a1 * q1) / (a0 + a1);
}

#ifdef __CUDA_ARCH__
// FP32 WENO3 in difference form (d1 = v1 - v2, d3 = v3 - v2), as weno5<float>.
template <>
__device__ __forceinline__ float weno3<float>(float v1, float v2, float v3) {
    const float eps = 1e-8f;
    const float d1 = __fsub_rn(v1, v2), d3 = __fsub_rn(v3, v2);
    const float b0 = __fmul_rn(d1, d1), b1 = __fmul_rn(d3, d3);
    const float tau = fabsf(__fsub_rn(b0, b1));
    const float r0 = __fdiv_rn(tau, __fadd_rn(b0, eps)), r1 = __fdiv_rn(tau, __fadd_rn(b1, eps));
    const float a0 = __fmul_rn(1.f / 3.f, fmaf(r0, r0, 1.f)), a1 = __fmul_rn(2.f / 3.f, fmaf(r1, r1, 1.f));
    const float num = fmaf(a0, __fmul_rn(-0.5f, d1), __fmul_rn(a1, __fmul_rn(0.5f, d3)));
    return __fadd_rn(__fdiv_rn(num, __fadd_rn(a0, a1)), v2);
}
#endif

}  // namespace obgc
