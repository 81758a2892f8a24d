// box.cu — batched BoxModel integration (src/BoxModel): one thread per independent 0-D model, the
// whole time loop in registers, RK3 exactly as BoxModel/timesteppers.jl:66-93 (compute every
// tracer's tendency, then U += dt (gamma G + zeta G-), G- = G).  Tracers without a tendency have
// G = 0 and are left unchanged.
#include "npd_device.cuh"

namespace obgc {

template <typename T>
__global__ void __launch_bounds__(128) box_kernel(obgc_npd_params p0, const obgc_npd_params* __restrict__ per_model,
                                                  int64_t n, double* __restrict__ state, const double* __restrict__ PAR,
                                                  double par_const, double dt_d, int nsteps, int record_every,
                                                  double* __restrict__ record) {
    const int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= n) return;
    const NPDParamsT<T> p = make_params<T>(per_model ? per_model[m] : p0);
    const T dt = T(dt_d);
    T v[OBGC_NUM_NAMED], G[OBGC_NUM_NAMED], Gm[OBGC_NUM_NAMED];
#pragma unroll
    for (int q = 0; q < OBGC_NUM_NAMED; q++) {
        v[q] = T(state[m * OBGC_NUM_NAMED + q]);
        Gm[q] = T(0);
    }
    int rec = 0;
    // Q10^(T/10): recomputed only when the box's temperature changes (it has no tendency, so never
    // within a run unless the caller changes it between runs) — the same value, without a pow per stage
    T Tlast = v[OBGC_T], Lt = p.q10 ? t_pow(p.Q10, Tlast / T(10)) : T(1);
    for (int s = 0; s < nsteps; s++) {
#pragma unroll
        for (int stg = 0; stg < 3; stg++) {
            const T par = PAR ? T(PAR[(int64_t)(3 * s + stg) * n + m]) : T(par_const);
#pragma unroll
            for (int q = 0; q < OBGC_NUM_NAMED; q++) G[q] = T(0);
            if (v[OBGC_T] != Tlast) {
                Tlast = v[OBGC_T];
                Lt = p.q10 ? t_pow(p.Q10, Tlast / T(10)) : T(1);
            }
            npd_tendencies<V_RUNTIME, T>(p, v, par, G, &Lt);
            const T g = T(rk3_gamma(stg)), z = T(rk3_zeta(stg));
#pragma unroll
            for (int q = 0; q < OBGC_NUM_NAMED; q++) {
                v[q] += stg == 0 ? dt * g * G[q] : dt * (g * G[q] + z * Gm[q]);
                Gm[q] = G[q];
            }
        }
        if (record && record_every > 0 && (s + 1) % record_every == 0) {
#pragma unroll
            for (int q = 0; q < OBGC_NUM_NAMED; q++) record[((int64_t)rec * n + m) * OBGC_NUM_NAMED + q] = (double)v[q];
            rec++;
        }
    }
#pragma unroll
    for (int q = 0; q < OBGC_NUM_NAMED; q++) state[m * OBGC_NUM_NAMED + q] = (double)v[q];
}

}  // namespace obgc

using namespace obgc;

extern "C" int obgc_box_run(const obgc_npd_params* p, const obgc_npd_params* per_model, int64_t n, double* state,
                            const double* PAR, double par_const, double t0, double dt, int32_t nsteps,
                            int32_t record_every, double* record, int32_t precision, void* stream) {
    (void)t0;
    if (!p || n < 0 || !state || nsteps < 0 || !(dt > 0) || (record_every > 0 && !record))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_box_run: bad argument");
    if (n == 0 || nsteps == 0) return OBGC_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = (int)((n + 127) / 128);
    if (precision == OBGC_PREC_F32)
        box_kernel<float><<<blocks, 128, 0, st>>>(*p, per_model, n, state, PAR, par_const, dt, nsteps, record_every, record);
    else if (precision == OBGC_PREC_F64)
        box_kernel<double><<<blocks, 128, 0, st>>>(*p, per_model, n, state, PAR, par_const, dt, nsteps, record_every, record);
    else
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_box_run: precision must be F32 or F64");
    OBGC_LAUNCHED("box_kernel");
    return OBGC_OK;
}
