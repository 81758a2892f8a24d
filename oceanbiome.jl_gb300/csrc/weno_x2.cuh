// weno_x2.cuh — two WENO5-Z reconstructions at once with Blackwell's packed FP32x2 arithmetic
// (fma/mul/add/sub .rn.f32x2, sm_100+): lane-local pairs (x face, y face) share one instruction
// stream, halving the FMA-pipe issue slots of the horizontal advection.  Same formula and
// rounding-to-nearest per element as weno5<float> (weno_device.cuh); only the four reciprocals per
// reconstruction stay scalar (MUFU).
#pragma once
#include "weno_device.cuh"

namespace obgc {

#ifdef __CUDA_ARCH__
typedef unsigned long long f32x2;

__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void up2(f32x2 v, float& lo, float& hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 splat2(float x) { return pk2(x, x); }
__device__ __forceinline__ f32x2 rcp2(f32x2 a) {
    float lo, hi;
    up2(a, lo, hi);
    return pk2(rcp_approx(lo), rcp_approx(hi));
}

// WENO5-Z of two upwind stencils (v1..v5 from far upwind to downwind), packed lo/hi, in the
// difference form of weno5<float> (d_k = v_k - v3).
__device__ __forceinline__ f32x2 weno5_x2(f32x2 v1, f32x2 v2, f32x2 v3, f32x2 v4, f32x2 v5) {
    const f32x2 c13 = splat2(2.f / 6.f), c76 = splat2(-7.f / 6.f);
    const f32x2 cm16 = splat2(-1.f / 6.f), c56 = splat2(5.f / 6.f);
    const f32x2 m2 = splat2(-2.f), m4 = splat2(-4.f);
    const f32x2 k1312 = splat2(13.f / 12.f), k14 = splat2(0.25f), one = splat2(1.f), eps = splat2(1e-8f);
    const f32x2 d1 = sub2(v1, v3), d2 = sub2(v2, v3), d4 = sub2(v4, v3), d5 = sub2(v5, v3);
    // candidate stencils relative to v3
    const f32x2 p0 = fma2(c13, d1, mul2(c76, d2));
    const f32x2 p1 = fma2(cm16, d2, mul2(c13, d4));
    const f32x2 p2 = fma2(c56, d4, mul2(cm16, d5));
    // smoothness indicators
    f32x2 a = fma2(m2, d2, d1);
    f32x2 b = fma2(m4, d2, d1);
    const f32x2 b0 = fma2(mul2(k1312, a), a, mul2(mul2(k14, b), b));
    a = add2(d2, d4);
    b = sub2(d2, d4);
    const f32x2 b1 = fma2(mul2(k1312, a), a, mul2(mul2(k14, b), b));
    a = fma2(m2, d4, d5);
    b = fma2(m4, d4, d5);
    const f32x2 b2 = fma2(mul2(k1312, a), a, mul2(mul2(k14, b), b));
    // tau = |b0 - b2| enters only through r_k^2: its sign changes no weight, so no abs (two ALU
    // instructions a pair)
    const f32x2 tau = sub2(b0, b2);
    const f32x2 r0 = mul2(tau, rcp2(add2(b0, eps)));
    const f32x2 r1 = mul2(tau, rcp2(add2(b1, eps)));
    const f32x2 r2 = mul2(tau, rcp2(add2(b2, eps)));
    const f32x2 a0 = mul2(splat2(0.1f), fma2(r0, r0, one));
    const f32x2 a1 = mul2(splat2(0.6f), fma2(r1, r1, one));
    const f32x2 a2 = mul2(splat2(0.3f), fma2(r2, r2, one));
    const f32x2 num = fma2(a0, p0, fma2(a1, p1, mul2(a2, p2)));
    return fma2(num, rcp2(add2(add2(a0, a1), a2)), v3);
}
#endif

}  // namespace obgc
