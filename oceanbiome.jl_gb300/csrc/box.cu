// box.cu — batched BoxModel integration (src/BoxModel): one thread per independent 0-D model, the
// whole time loop in registers, RK3 exactly as BoxModel/timesteppers.jl:66-93 (compute every
// tracer's tendency, then U += dt (gamma G + zeta G-), G- = G).  Tracers without a tendency have
// G = 0 and are left unchanged.
#include <cstring>
#include "npd_device.cuh"

namespace obgc {

// Prescribed tracers and forcings by tracer name: bit r of pmask / fmask marks tracer r, whose
// series is presc[pslot[r]] / frc[fslot[r]] (the name loops unroll, so the state stays in registers).
struct BoxDrv {
    uint32_t pmask, fmask;
    int8_t pslot[OBGC_NUM_NAMED], fslot[OBGC_NUM_NAMED];
    const double* presc[OBGC_BOX_MAX_DRIVERS];
    const double* frc[OBGC_BOX_MAX_DRIVERS];
};

template <typename T>
__device__ __forceinline__ void box_prescribe(const BoxDrv& d, T* v, int64_t row) {
#pragma unroll
    for (int r = 0; r < OBGC_NUM_NAMED; r++)
        if ((d.pmask >> r) & 1u) v[r] = T(d.presc[d.pslot[r]][row]);
}

template <typename T, bool DRV>
__global__ void __launch_bounds__(128) box_kernel(obgc_npd_params p0, const obgc_npd_params* __restrict__ per_model,
                                                  int64_t n, double* __restrict__ state, const double* __restrict__ PAR,
                                                  double par_const, double dt_d, int nsteps, int record_every,
                                                  double* __restrict__ record, const __grid_constant__ BoxDrv drv) {
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
            const int64_t row = (int64_t)(3 * s + stg) * n + m;
            const T par = PAR ? T(PAR[row]) : T(par_const);
            if (DRV && drv.pmask) box_prescribe(drv, v, row);   // update_state! at the stage time
#pragma unroll
            for (int q = 0; q < OBGC_NUM_NAMED; q++) G[q] = T(0);
            if (v[OBGC_T] != Tlast) {
                Tlast = v[OBGC_T];
                Lt = p.q10 ? t_pow(p.Q10, Tlast / T(10)) : T(1);
            }
            npd_tendencies<V_RUNTIME, T>(p, v, par, G, &Lt);
            if (DRV && drv.fmask) {
#pragma unroll
                for (int r = 0; r < OBGC_NUM_NAMED; r++)
                    if ((drv.fmask >> r) & 1u) G[r] += T(drv.frc[drv.fslot[r]][row]);
            }
            const T g = T(rk3_gamma(stg)), z = T(rk3_zeta(stg));
#pragma unroll
            for (int q = 0; q < OBGC_NUM_NAMED; q++) {
                v[q] += stg == 0 ? dt * g * G[q] : dt * (g * G[q] + z * Gm[q]);
                Gm[q] = G[q];
            }
        }
        if (DRV && drv.pmask) box_prescribe(drv, v, (int64_t)(3 * (s + 1)) * n + m);   // update_state! at the step's end
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

extern "C" int obgc_box_run_drivers(const obgc_npd_params* p, const obgc_npd_params* per_model, int64_t n, double* state,
                                    const obgc_box_drivers* d, double t0, double dt, int32_t nsteps, int32_t record_every,
                                    double* record, int32_t precision, void* stream) {
    (void)t0;
    if (!p || !d || n < 0 || !state || nsteps < 0 || !(dt > 0) || (record_every > 0 && !record) || d->n_prescribed < 0 ||
        d->n_prescribed > OBGC_BOX_MAX_DRIVERS || d->n_forced < 0 || d->n_forced > OBGC_BOX_MAX_DRIVERS)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_box_run: bad argument");
    BoxDrv drv;
    std::memset(&drv, 0, sizeof(drv));
    for (int q = 0; q < d->n_prescribed; q++) {
        const int r = d->prescribed_names[q];
        if (r < 0 || r >= OBGC_NUM_NAMED || !d->prescribed[q] || ((drv.pmask >> r) & 1u))
            return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_box_run: bad prescribed tracer");
        drv.pmask |= 1u << r;
        drv.pslot[r] = (int8_t)q;
        drv.presc[q] = d->prescribed[q];
    }
    for (int q = 0; q < d->n_forced; q++) {
        const int r = d->forced_names[q];
        if (r < 0 || r >= OBGC_NUM_NAMED || !d->forcing[q] || ((drv.fmask >> r) & 1u))
            return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_box_run: bad forced tracer");
        drv.fmask |= 1u << r;
        drv.fslot[r] = (int8_t)q;
        drv.frc[q] = d->forcing[q];
    }
    if (n == 0 || nsteps == 0) return OBGC_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = (int)((n + 127) / 128);
    // the driver-free instantiation keeps the plain run free of the per-stage driver checks
    const bool any = drv.pmask != 0u || drv.fmask != 0u;
    if (precision == OBGC_PREC_F32) {
        if (any) box_kernel<float, true><<<blocks, 128, 0, st>>>(*p, per_model, n, state, d->PAR, d->par_constant, dt, nsteps,
                                                                 record_every, record, drv);
        else box_kernel<float, false><<<blocks, 128, 0, st>>>(*p, per_model, n, state, d->PAR, d->par_constant, dt, nsteps,
                                                              record_every, record, drv);
    } else if (precision == OBGC_PREC_F64) {
        if (any) box_kernel<double, true><<<blocks, 128, 0, st>>>(*p, per_model, n, state, d->PAR, d->par_constant, dt, nsteps,
                                                                  record_every, record, drv);
        else box_kernel<double, false><<<blocks, 128, 0, st>>>(*p, per_model, n, state, d->PAR, d->par_constant, dt, nsteps,
                                                               record_every, record, drv);
    } else {
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_box_run: precision must be F32 or F64");
    }
    OBGC_LAUNCHED("box_kernel");
    return OBGC_OK;
}

extern "C" int obgc_box_run(const obgc_npd_params* p, const obgc_npd_params* per_model, int64_t n, double* state,
                            const double* PAR, double par_const, double t0, double dt, int32_t nsteps,
                            int32_t record_every, double* record, int32_t precision, void* stream) {
    obgc_box_drivers d;
    std::memset(&d, 0, sizeof(d));
    d.PAR = PAR;
    d.par_constant = par_const;
    return obgc_box_run_drivers(p, per_model, n, state, &d, t0, dt, nsteps, record_every, record, precision, stream);
}
