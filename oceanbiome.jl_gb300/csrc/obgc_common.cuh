// obgc_common.cuh — status handling, launch accounting and small numeric helpers shared by every
// translation unit of libobgc.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include "../../include/obgc.h"

namespace obgc {

// Last error text of the calling host thread (obgc_last_error_message).
void set_error(const std::string& msg);
int fail(int status, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);
// Count of kernels launched by this library in this process (obgc_kernel_launch_count).
void count_launches(int64_t n);

#define OBGC_CUDA(call)                                                                   \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) return ::obgc::cuda_fail(e_, #call);                       \
    } while (0)

#define OBGC_LAUNCHED(where)                                                              \
    do {                                                                                  \
        ::obgc::count_launches(1);                                                        \
        cudaError_t e_ = cudaGetLastError();                                              \
        if (e_ != cudaSuccess) return ::obgc::cuda_fail(e_, where);                       \
    } while (0)

inline bool valid_grid(const obgc_grid* g) {
    if (!g || g->Nx < 1 || g->Ny < 1 || g->Nz < 1) return false;
    if (g->stride_j < g->Nx || g->stride_k < g->stride_j * (int64_t)g->Ny) return false;
    if (!(g->Lz > 0)) return false;
    return true;
}

// Julia's eps(x): spacing of |x| at its binade; eps(0) = smallest subnormal.
__host__ __device__ inline double jl_eps(double x) {
    double a = fabs(x);
    if (a < 2.2250738585072014e-308) return 4.9406564584124654e-324;
    int e;
    frexp(a, &e);
    return ldexp(2.220446049250313e-16, e - 1);
}
__host__ __device__ inline float jl_eps(float x) {
#ifdef __CUDA_ARCH__
    unsigned e = (__float_as_uint(x) >> 23) & 0xffu;
    if (e >= 24u) return __uint_as_float((e - 23u) << 23);
    if (e == 0u) return __uint_as_float(1u);
    return __uint_as_float(1u << (e - 1u));
#else
    float a = fabsf(x);
    if (a < 1.17549435e-38f) return 1.4e-45f;
    int e;
    frexpf(a, &e);
    return ldexpf(1.1920929e-7f, e - 1);
#endif
}
// eps(0.0) in the working precision (the reference adds eps(0.0) to guard 0/0).
template <typename T> __host__ __device__ inline T tiny();
template <> __host__ __device__ inline double tiny<double>() { return 4.9406564584124654e-324; }
template <> __host__ __device__ inline float tiny<float>() { return 1.40129846e-45f; }

template <typename T> __host__ __device__ inline T t_exp(T x);
template <> __host__ __device__ inline double t_exp(double x) { return exp(x); }
template <> __host__ __device__ inline float t_exp(float x) { return expf(x); }
template <typename T> __host__ __device__ inline T t_pow(T x, T y);
template <> __host__ __device__ inline double t_pow(double x, double y) { return pow(x, y); }
template <> __host__ __device__ inline float t_pow(float x, float y) { return powf(x, y); }
template <typename T> __host__ __device__ inline T t_sqrt(T x);
template <> __host__ __device__ inline double t_sqrt(double x) { return sqrt(x); }
template <> __host__ __device__ inline float t_sqrt(float x) { return sqrtf(x); }
template <typename T> __host__ __device__ inline T t_abs(T x) { return x < T(0) ? -x : x; }
template <typename T> __host__ __device__ inline T t_max0(T x) { return x > T(0) ? x : (x == x ? T(0) : x); }

// Oceananigans RungeKutta3 coefficients: gamma, zeta and the stage start times (fractions of dt).
__host__ __device__ constexpr double rk3_gamma(int s) { return s == 0 ? 8.0 / 15.0 : (s == 1 ? 5.0 / 12.0 : 3.0 / 4.0); }
__host__ __device__ constexpr double rk3_zeta(int s) { return s == 0 ? 0.0 : (s == 1 ? -17.0 / 60.0 : -5.0 / 12.0); }
__host__ __device__ constexpr double rk3_c(int s) { return s == 0 ? 0.0 : (s == 1 ? 8.0 / 15.0 : 2.0 / 3.0); }

}  // namespace obgc
