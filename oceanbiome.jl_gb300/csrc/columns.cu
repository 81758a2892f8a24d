// columns.cu — packed, shared-memory-resident stepping of many uneven 1-D columns.
//
// One thread block owns a "pack" of whole columns (first-fit by cell count) and keeps their
// state, previous-stage tendencies, PAR, sinking fluxes, diffusivities and tridiagonal factors in
// shared memory for every step of a launch, so a launch touches HBM only to load and store the
// state once.  Per RK3 stage:
//   1. TwoBand PAR: one warp per column, a warp-shuffle prefix sum of the chlorophyll terms down
//      the column in chunks of 32 levels (2band.jl:15-32).
//   2. Sinking face fluxes (WENO5 with the wall order reduction of the 3-D path) of the two
//      drifting tracers (NPZD: P, D; LOBSTER: sPOM, bPOM).
//   2b. With the CO2 gas exchange (LOBSTER columns): one thread per column takes the air-sea flux
//      from the surface DIC and Alk and the column's T and S (FP64 pCO2 solve).
//   3. Every cell: BGC tendency + sinking divergence (+ the surface flux / dz on DIC's top cell),
//      RK3 update U += dt (gamma G + zeta G-).
//   4. Vertically implicit diffusion (I - dt_s d/dz kappa d/dz) U = U*, dt_s = (gamma + zeta) dt,
//      zero-flux walls: one Thomas solve per (column, tracer) with factors precomputed per stage.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>
#include "columns_engine.h"
#include "gas_device.cuh"
#include "negatives.cuh"
#include "step_kernel.cuh"

namespace obgc {

// TS: state precision (shared-memory state, RK3 accumulation, diffusion solve); TC: compute
// precision of the light, sinking fluxes and BGC tendencies.
template <typename TS, typename TC>
struct ColArgs {
    ColSlot<TS>* slots;         // steps_left / steps_done are advanced in place
    const int32_t* pack_slots;
    const ColPack* packs;
    TS* state;
    const TS* kappa;
    NPDParamsT<TC> bgc;
    TwoBandT<TC> light;
    TC w0A, w0B;                // sinking speeds of the two window tracers (m/s, positive down)
    int open_bottom;
    int max_steps;
    int cap;
    NegativesSpec neg;          // modifier applied to the initial state and after every stage
    int co2;                    // CO2 gas exchange on DIC (LOBSTER columns)
    obgc_gas_exchange gas;
};

template <typename TS, typename TC, int NT>
__host__ __device__ constexpr size_t col_smem_bytes(int cap) {
    return sizeof(TS) * ((size_t)NT * cap + (cap + COL_MAXC) + 6 * (size_t)cap + 8 * COL_MAXC) +
           sizeof(TC) * ((size_t)NT * cap + cap + 2 * (size_t)(cap + COL_MAXC)) + sizeof(int64_t) * COL_MAXC +
           sizeof(int) * 6 * COL_MAXC + sizeof(short) * ((size_t)2 * cap + COL_MAXC);
}

// The CO2 condition's per-column state after the layout above (engines with the condition only):
// the cached T/S constants and the [H+] each column's solve restarts from.
template <typename TS, typename TC, int NT>
__host__ __device__ constexpr size_t col_co2_offset(int cap) {
    return (col_smem_bytes<TS, TC, NT>(cap) + 15) / 16 * 16;
}
constexpr size_t COL_CO2_BYTES = (sizeof(Co2Column) + sizeof(double)) * COL_MAXC;

template <typename T>
__device__ __forceinline__ T sink_w(T w0, int open_bottom, int f, int Nz) {
    // setup_velocity_fields (sinking_velocity_fields.jl:10-35); the surface face stays zero
    if (f >= Nz) return T(0);
    return -w0 * (open_bottom ? T(1) : (T(1) - t_exp(T(-f) / T(2))));
}

template <int V, int NT, typename TS, typename TC>
__global__ void __launch_bounds__(512, 1) column_kernel(const __grid_constant__ ColArgs<TS, TC> a) {
    constexpr int SP = slot_of_P(V);
    constexpr int WA = V == V_NPZD ? 1 : 4, WB = V == V_NPZD ? 4 : 5;
    constexpr int SALK = V == V_NPZD ? -1 : 8, SDIC = V == V_NPZD ? -1 : 7;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const ColPack pk = a.packs[blockIdx.x];
    const int ncol = pk.count, cells = pk.cells, cap = a.cap;
    const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarp = nth >> 5;

    TS* U = reinterpret_cast<TS*>(smem_raw);
    TS* kap = U + NT * cap;                  // faces of each column
    TS* th = kap + (cap + COL_MAXC);         // [3 stages][cp, inverse pivot][cap]
    TS* cdz = th + 6 * cap;
    TS* cdt = cdz + COL_MAXC;
    TS* cP0 = cdt + COL_MAXC;
    TS* cmu = cP0 + COL_MAXC;
    TS* cpa = cmu + COL_MAXC;
    TS* cr = cpa + COL_MAXC;                 // the stage's air-sea flux of each column
    TS* cT = cr + COL_MAXC;                  // surface T and S of each column
    TS* cS = cT + COL_MAXC;
    TC* Gm = reinterpret_cast<TC*>(cS + COL_MAXC);
    TC* PAR = Gm + NT * cap;
    TC* F = PAR + cap;                       // [2][cap + COL_MAXC] sinking fluxes
    int64_t* cbase = reinterpret_cast<int64_t*>(F + 2 * (cap + COL_MAXC));
    int* coff = reinterpret_cast<int*>(cbase + COL_MAXC);
    int* cnz = coff + COL_MAXC;
    int* cst = cnz + COL_MAXC;
    int* cdone = cst + COL_MAXC;
    int* cps = cdone + COL_MAXC;
    int* cpk = cps + COL_MAXC;
    short* colid = reinterpret_cast<short*>(cpk + COL_MAXC);
    short* fcol = colid + cap;
    Co2Column* cco2 = reinterpret_cast<Co2Column*>(smem_raw + col_co2_offset<TS, TC, NT>(cap));
    double* cH = reinterpret_cast<double*>(cco2 + COL_MAXC);

    if (tid < ncol) {
        const ColSlot<TS> sl = a.slots[a.pack_slots[pk.first + tid]];
        cbase[tid] = sl.cell_off;
        cnz[tid] = sl.Nz;
        cst[tid] = min(sl.steps_left, a.max_steps);
        cdone[tid] = sl.steps_done;
        cps[tid] = sl.pulse_step;
        cpk[tid] = sl.pulse_k;
        cdz[tid] = sl.dz;
        cdt[tid] = sl.dt;
        cP0[tid] = sl.PAR0;
        cmu[tid] = sl.mu0;
        cpa[tid] = sl.pulse_amount;
        cT[tid] = sl.temp;
        cS[tid] = sl.sal;
        cr[tid] = TS(0);
        if constexpr (SDIC >= 0) {
            if (a.co2) {
                co2_column_prepare(a.gas, double(sl.temp), double(sl.sal), a.gas.wind_speed, cco2[tid]);
                cH[tid] = exp(-2.302585092994046 * a.gas.carbon.initial_pH_guess);
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        int o = 0;
        for (int c = 0; c < ncol; c++) { coff[c] = o; o += cnz[c]; }
    }
    __syncthreads();
    for (int c = warp; c < ncol; c += nwarp) {
        for (int k = lane; k < cnz[c]; k += 32) colid[coff[c] + k] = (short)c;
        for (int f = lane; f <= cnz[c]; f += 32) fcol[coff[c] + c + f] = (short)c;
    }
    __syncthreads();
    // load state [NT][Nz] and face diffusivities of every column
    for (int i = tid; i < cells; i += nth) {
        const int c = colid[i], k = i - coff[c], Nz = cnz[c];
        const TS* src = a.state + cbase[c] * NT;
#pragma unroll
        for (int t = 0; t < NT; t++) {
            U[t * cap + i] = src[(int64_t)t * Nz + k];
            Gm[t * cap + i] = TC(0);
        }
    }
    for (int fi = tid; fi < cells + ncol; fi += nth) {
        const int c = fcol[fi], f = fi - coff[c] - c;
        kap[fi] = a.kappa[cbase[c] + f];
    }
    __syncthreads();
    // tridiagonal factors of every (column, stage)
    for (int it = tid; it < 3 * ncol; it += nth) {
        const int c = it / 3, st = it - 3 * c, Nz = cnz[c];
        const TS r = TS(rk3_gamma(st) + rk3_zeta(st)) * cdt[c] / (cdz[c] * cdz[c]);
        const TS* kf = kap + coff[c] + c;
        TS* cp = th + (2 * st) * cap + coff[c];
        TS* idn = th + (2 * st + 1) * cap + coff[c];
        TS cprev = TS(0);
        for (int k = 0; k < Nz; k++) {
            const TS lo = k > 0 ? -r * kf[k] : TS(0);
            const TS up = k < Nz - 1 ? -r * kf[k + 1] : TS(0);
            const TS di = TS(1) - lo - up;
            const TS den = k == 0 ? di : di - lo * cprev;
            cprev = up / den;
            cp[k] = cprev;
            idn[k] = TS(1) / den;
        }
    }
    __syncthreads();
    if (a.neg.mode != OBGC_NEGATIVES_NONE) {
        // update_state! before the first step of a column (set! / iteration 0)
        for (int i = tid; i < cells; i += nth) {
            const int c = colid[i];
            if (cdone[c] == 0 && cst[c] > 0) negatives_cell<TS>(a.neg, [&](int q) -> TS& { return U[q * cap + i]; });
        }
        __syncthreads();
    }

    for (int s = 0; s < a.max_steps; s++) {
        if (SALK >= 0 && tid < ncol && s < cst[tid] && cdone[tid] + s == cps[tid] && cpk[tid] >= 0 && cpk[tid] < cnz[tid])
            U[SALK * cap + coff[tid] + cpk[tid]] += cpa[tid];
        __syncthreads();
#pragma unroll 1
        for (int st = 0; st < 3; st++) {
            // 1. PAR: warp-shuffle scan down each column
            for (int c = warp; c < ncol; c += nwarp) {
                if (s >= cst[c]) continue;
                const int Nz = cnz[c], base = coff[c];
                const TC dz = TC(cdz[c]), P0 = TC(cP0[c]);
                TC carry_r = TC(0), carry_b = TC(0);
                for (int k0 = Nz - 1; k0 >= 0; k0 -= 32) {
                    const int k = k0 - lane;
                    TC fr = TC(0), fb = TC(0);
                    if (k >= 0) twoband_terms(a.light, TC(U[SP * cap + base + k]), fr, fb);
                    TC sr = fr, sb = fb;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const TC yr = __shfl_up_sync(0xffffffffu, sr, o), yb = __shfl_up_sync(0xffffffffu, sb, o);
                        if (lane >= o) { sr += yr; sb += yb; }
                    }
                    if (k >= 0) {
                        const TC z = -TC(Nz) * dz + (TC(k) + TC(0.5)) * dz;
                        PAR[base + k] = twoband_par(a.light, P0, z, dz, carry_r + (sr - fr), carry_b + (sb - fb), fr, fb);
                    }
                    carry_r += __shfl_sync(0xffffffffu, sr, 31);
                    carry_b += __shfl_sync(0xffffffffu, sb, 31);
                }
            }
            // 2. sinking fluxes through every face of every column
            for (int fi = tid; fi < cells + ncol; fi += nth) {
                const int c = fcol[fi], f = fi - coff[c] - c, Nz = cnz[c];
                if (s >= cst[c]) continue;
                const TS* xa = U + WA * cap + coff[c];
                const TS* xb = U + WB * cap + coff[c];
                TC w[6];
                if (a.w0A != TC(0)) {
#pragma unroll
                    for (int m = 0; m < 6; m++) w[m] = TC(xa[min(max(f - 3 + m, 0), Nz - 1)]);
                    F[fi] = window_face_flux(w[0], w[1], w[2], w[3], w[4], w[5], f, Nz, sink_w(a.w0A, a.open_bottom, f, Nz));
                } else {
                    F[fi] = TC(0);
                }
                if (a.w0B != TC(0)) {
#pragma unroll
                    for (int m = 0; m < 6; m++) w[m] = TC(xb[min(max(f - 3 + m, 0), Nz - 1)]);
                    F[cap + COL_MAXC + fi] = window_face_flux(w[0], w[1], w[2], w[3], w[4], w[5], f, Nz,
                                                              sink_w(a.w0B, a.open_bottom, f, Nz));
                } else {
                    F[cap + COL_MAXC + fi] = TC(0);
                }
            }
            // 2b. air-sea CO2 flux of every column from its surface cell (gas_exchange.jl:26-39)
            if constexpr (SDIC >= 0) {
                if (a.co2 && tid < ncol && s < cst[tid]) {
                    const int top = coff[tid] + cnz[tid] - 1;
                    cr[tid] = TS(co2_column_flux(a.gas, cco2[tid], double(U[SDIC * cap + top]), double(U[SALK * cap + top]),
                                                 a.gas.air_concentration, cH[tid]));
                }
            }
            __syncthreads();
            // 3. BGC + sinking divergence + RK3 update of every cell (increment in TC, sum in TS)
            const TC gam = TC(rk3_gamma(st)), zet = TC(rk3_zeta(st));
            for (int i = tid; i < cells; i += nth) {
                const int c = colid[i];
                if (s >= cst[c]) continue;
                const int k = i - coff[c], fi = coff[c] + c + k;
                TC vals[OBGC_NUM_NAMED], g[OBGC_NUM_NAMED];
#pragma unroll
                for (int n = 0; n < OBGC_NUM_NAMED; n++) { vals[n] = TC(0); g[n] = TC(0); }
#pragma unroll
                for (int q = 0; q < NT; q++) vals[slot_name(V, q)] = TC(U[q * cap + i]);
                NPDParamsT<TC> pc = a.bgc;
                if (cmu[c] > TS(0)) pc.mu0 = TC(cmu[c]);
                npd_tendencies<V, TC>(pc, vals, PAR[i], g);
                const TC idz = TC(1) / TC(cdz[c]), dt = TC(cdt[c]);
#pragma unroll
                for (int q = 0; q < NT; q++) {
                    TC G = g[slot_name(V, q)];
                    if (q == WA) G -= (F[fi + 1] - F[fi]) * idz;
                    if (q == WB) G -= (F[cap + COL_MAXC + fi + 1] - F[cap + COL_MAXC + fi]) * idz;
                    if (q == SDIC && k == cnz[c] - 1) G -= TC(cr[c]) * idz;   // zero without the condition
                    const TC upd = st == 0 ? dt * gam * G : dt * (gam * G + zet * Gm[q * cap + i]);
                    U[q * cap + i] += TS(upd);
                    Gm[q * cap + i] = G;
                }
            }
            __syncthreads();
            // 4. implicit vertical diffusion: one warp per (column, tracer).  The two Thomas sweeps are
            // first-order linear recurrences, d_k = a_k d_(k-1) + b_k forward and x_k = -cp_k x_(k+1)
            // + d_k backward, so each 32-level chunk composes its lanes' affine maps with a shuffle
            // scan and applies the composite to the carry from the chunk before.
            for (int it = warp; it < ncol * NT; it += nwarp) {
                const int c = it / NT, q = it - c * NT;
                if (s >= cst[c]) continue;
                const int Nz = cnz[c];
                const TS r = TS(rk3_gamma(st) + rk3_zeta(st)) * cdt[c] / (cdz[c] * cdz[c]);
                const TS* kf = kap + coff[c] + c;
                const TS* cp = th + (2 * st) * cap + coff[c];
                const TS* idn = th + (2 * st + 1) * cap + coff[c];
                TS* x = U + q * cap + coff[c];
                TS carry = TS(0);
                for (int k0 = 0; k0 < Nz; k0 += 32) {
                    const int k = k0 + lane;
                    TS A = TS(1), B = TS(0);   // identity past the column
                    if (k < Nz) {
                        A = k == 0 ? TS(0) : r * kf[k] * idn[k];
                        B = x[k] * idn[k];
                    }
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const TS Ap = __shfl_up_sync(0xffffffffu, A, o), Bp = __shfl_up_sync(0xffffffffu, B, o);
                        if (lane >= o) { B = A * Bp + B; A = A * Ap; }
                    }
                    const TS d = A * carry + B;
                    if (k < Nz) x[k] = d;
                    carry = __shfl_sync(0xffffffffu, d, 31);
                }
                __syncwarp();
                carry = x[Nz - 1];
                for (int k0 = 0; k0 < Nz - 1; k0 += 32) {
                    const int k = Nz - 2 - (k0 + lane);
                    TS A = TS(1), B = TS(0);
                    if (k >= 0) {
                        A = -cp[k];
                        B = x[k];
                    }
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const TS Ap = __shfl_up_sync(0xffffffffu, A, o), Bp = __shfl_up_sync(0xffffffffu, B, o);
                        if (lane >= o) { B = A * Bp + B; A = A * Ap; }
                    }
                    const TS v = A * carry + B;
                    if (k >= 0) x[k] = v;
                    carry = __shfl_sync(0xffffffffu, v, 31);
                }
                __syncwarp();
            }
            __syncthreads();
            // 5. update_state! after the substep: the negative-tracer modifier
            if (a.neg.mode != OBGC_NEGATIVES_NONE) {
                for (int i = tid; i < cells; i += nth) {
                    if (s >= cst[colid[i]]) continue;
                    negatives_cell<TS>(a.neg, [&](int q) -> TS& { return U[q * cap + i]; });
                }
                __syncthreads();
            }
        }
    }
    // store the state back and count the steps taken
    for (int i = tid; i < cells; i += nth) {
        const int c = colid[i], k = i - coff[c], Nz = cnz[c];
        TS* dst = a.state + cbase[c] * NT;
#pragma unroll
        for (int t = 0; t < NT; t++) dst[(int64_t)t * Nz + k] = U[t * cap + i];
    }
    if (tid < ncol) {
        ColSlot<TS>& sl = a.slots[a.pack_slots[pk.first + tid]];
        sl.steps_left -= cst[tid];
        sl.steps_done += cst[tid];
    }
}

int required_tracers(const obgc_npd_params* p, int32_t* names);
bool drift_speed(const obgc_npd_params* p, int name, double* w0);
bool valid_gas(const obgc_gas_exchange* g);

}  // namespace obgc

using namespace obgc;

namespace obgc {
namespace cols {

template <typename TS, typename TC>
void* column_kernel_ptr(int V) {
    return V == V_NPZD ? (void*)column_kernel<V_NPZD, 5, TS, TC> : (void*)column_kernel<V_LOBSTER_C, 9, TS, TC>;
}

size_t smem_for(const obgc_columns* e, int cap);

// Dynamic shared memory above 48 KiB must be opted into before a launch (and before a capture).
int prepare_launch(obgc_columns* e, int cap) {
    void* fn = e->prec == OBGC_PREC_F32 ? column_kernel_ptr<float, float>(e->V)
             : e->prec == OBGC_PREC_F64 ? column_kernel_ptr<double, double>(e->V)
                                        : column_kernel_ptr<double, float>(e->V);
    const cudaError_t err = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_for(e, cap));
    if (err != cudaSuccess) return cuda_fail(err, "cudaFuncSetAttribute(column_kernel)");
    return OBGC_OK;
}

template <typename TS, typename TC>
int launch_columns(obgc_columns* e, int npacks, int max_steps, int threads, int cap, cudaStream_t st) {
    ColArgs<TS, TC> a;
    std::memset(&a, 0, sizeof(a));
    a.slots = static_cast<ColSlot<TS>*>(e->d_slots);
    a.pack_slots = e->d_pack_slots;
    a.packs = e->d_packs;
    a.state = static_cast<TS*>(e->state);
    a.kappa = static_cast<const TS*>(e->kappa);
    a.bgc = make_params<TC>(e->desc.npd);
    a.light = make_twoband<TC>(e->desc.light);
    a.w0A = TC(e->w0A);
    a.w0B = TC(e->w0B);
    a.open_bottom = e->desc.npd.open_bottom;
    a.max_steps = max_steps;
    a.cap = cap;
    a.neg = e->neg;
    a.co2 = e->desc.gas_exchange;
    a.gas = e->desc.gas;
    const size_t smem = smem_for(e, cap);
    if (e->V == V_NPZD) column_kernel<V_NPZD, 5, TS, TC><<<npacks, threads, smem, st>>>(a);
    else column_kernel<V_LOBSTER_C, 9, TS, TC><<<npacks, threads, smem, st>>>(a);
    OBGC_LAUNCHED("column_kernel");
    return OBGC_OK;
}

int launch_any(obgc_columns* e, int npacks, int max_steps, int threads, int cap, cudaStream_t st) {
    if (e->prec == OBGC_PREC_F32) return launch_columns<float, float>(e, npacks, max_steps, threads, cap, st);
    if (e->prec == OBGC_PREC_F64) return launch_columns<double, double>(e, npacks, max_steps, threads, cap, st);
    return launch_columns<double, float>(e, npacks, max_steps, threads, cap, st);
}

size_t smem_for(const obgc_columns* e, int cap) {
    const bool npzd = e->V == V_NPZD;
    if (npzd) {
        if (e->prec == OBGC_PREC_F32) return col_smem_bytes<float, float, 5>(cap);
        if (e->prec == OBGC_PREC_F64) return col_smem_bytes<double, double, 5>(cap);
        return col_smem_bytes<double, float, 5>(cap);
    }
    // LOBSTER: the CO2 condition's per-column state follows the common layout
    const size_t co2 = e->desc.gas_exchange ? COL_CO2_BYTES : 0;
    if (e->prec == OBGC_PREC_F32) return (co2 ? col_co2_offset<float, float, 9>(cap) : col_smem_bytes<float, float, 9>(cap)) + co2;
    if (e->prec == OBGC_PREC_F64)
        return (co2 ? col_co2_offset<double, double, 9>(cap) : col_smem_bytes<double, double, 9>(cap)) + co2;
    return (co2 ? col_co2_offset<double, float, 9>(cap) : col_smem_bytes<double, float, 9>(cap)) + co2;
}

// First-fit decreasing packing of the live columns into packs of `cap` cells, written to staging
// buffer b.
int build_packs(obgc_columns* e, int cap, int b) {
    std::vector<int> live;
    for (int s = 0; s < (int)e->slots.size(); s++)
        if (e->slots[s].live && e->slots[s].steps_left > 0) live.push_back(s);
    std::stable_sort(live.begin(), live.end(), [&](int x, int y) { return e->slots[x].Nz > e->slots[y].Nz; });
    std::vector<std::vector<int>> packs;
    std::vector<int> fill;
    for (int s : live) {
        const int nz = e->slots[s].Nz;
        int p = -1;
        for (int q = 0; q < (int)packs.size(); q++)
            if (fill[q] + nz <= cap && (int)packs[q].size() < COL_MAXC) { p = q; break; }
        if (p < 0) { packs.emplace_back(); fill.push_back(0); p = (int)packs.size() - 1; }
        packs[p].push_back(s);
        fill[p] += nz;
    }
    int n = 0;
    for (int q = 0; q < (int)packs.size(); q++) {
        e->h_packs[b][q] = {n, (int)packs[q].size(), fill[q], 0};
        for (int s : packs[q]) e->h_pack_slots[b][n++] = s;
    }
    return (int)packs.size();
}

// Convert the host slot table to the kernel's precision; returns the slots in use (highest live + 1).
template <typename T>
int stage_slots(obgc_columns* e, int b) {
    ColSlot<T>* h = static_cast<ColSlot<T>*>(e->h_slots[b]);
    int n = 0;
    for (size_t s = 0; s < e->slots.size(); s++)
        if (e->slots[s].live) n = (int)s + 1;
    for (int s = 0; s < n; s++) {
        const ColSlot<double>& d = e->slots[s];
        ColSlot<T> o;
        o.cell_off = d.cell_off; o.Nz = d.Nz; o.steps_left = d.steps_left; o.steps_done = d.steps_done;
        o.pulse_step = d.pulse_step; o.pulse_k = d.pulse_k; o.live = d.live;
        o.dz = T(d.dz); o.dt = T(d.dt); o.PAR0 = T(d.PAR0); o.mu0 = T(d.mu0); o.pulse_amount = T(d.pulse_amount);
        o.temp = T(d.temp); o.sal = T(d.sal); o.pad = T(0);
        h[s] = o;
    }
    return n;
}

int drain(obgc_columns* e) {
    if (e->pending) OBGC_CUDA(cudaStreamSynchronize(e->last_stream));
    e->pending = false;
    return OBGC_OK;
}

int stage_tables(obgc_columns* e, int cap, cudaStream_t st) {
    // the device tables are read by the kernels already queued: another stream must wait for them
    if (e->pending && st != e->last_stream) {
        const int rc = drain(e);
        if (rc != OBGC_OK) return -rc;
    }
    const int b = e->tb ^ 1;
    if (e->tables_used[b]) {
        const cudaError_t w = cudaEventSynchronize(e->tables_ev[b]);
        if (w != cudaSuccess) return -cuda_fail(w, "cudaEventSynchronize(column tables)");
    }
    const int npacks = build_packs(e, cap, b);
    if (npacks == 0) return 0;
    const size_t sb = e->ts == 4 ? sizeof(ColSlot<float>) : sizeof(ColSlot<double>);
    const int nslots = e->ts == 4 ? stage_slots<float>(e, b) : stage_slots<double>(e, b);
    const int nlive = e->h_packs[b][npacks - 1].first + e->h_packs[b][npacks - 1].count;
    e->last_stream = st;
    e->pending = true;
    cudaError_t err = cudaMemcpyAsync(e->d_slots, e->h_slots[b], sb * nslots, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(e->d_pack_slots, e->h_pack_slots[b], sizeof(int32_t) * nlive, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess)
        err = cudaMemcpyAsync(e->d_packs, e->h_packs[b], sizeof(ColPack) * npacks, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) err = cudaEventRecord(e->tables_ev[b], st);
    if (err != cudaSuccess) return -cuda_fail(err, "cudaMemcpyAsync(column tables)");
    e->tables_used[b] = true;
    e->tb = b;
    return npacks;
}

// Host mirror of the kernel's bookkeeping: every unfinished column took min(steps, left) steps.
void account_steps(obgc_columns* e, int steps) {
    for (auto& s : e->slots) {
        if (!s.live || s.steps_left <= 0) continue;
        const int done = std::min(steps, s.steps_left);
        s.steps_left -= done;
        s.steps_done += done;
    }
}

int advance_with(obgc_columns* e, int max_steps, int threads, int cap, cudaStream_t st, bool update_host) {
    const int npacks = stage_tables(e, cap, st);
    if (npacks <= 0) return -npacks;
    int rc;
    e->last_stream = st;
    e->pending = true;
    rc = prepare_launch(e, cap);
    if (rc != OBGC_OK) return rc;
    rc = launch_any(e, npacks, max_steps, threads, cap, st);
    if (rc != OBGC_OK) return rc;
    if (update_host) account_steps(e, max_steps);
    return OBGC_OK;
}

int reserve_column(obgc_columns* e, const obgc_column_spec* sp, int64_t* slot) {
    if (e->free_slots.empty()) return fail(OBGC_ERR_BUSY, "no free column slot");
    const int64_t need = sp->Nz + 1;   // Nz state cells and Nz+1 faces share the block
    auto it = e->free_cells.begin();
    for (; it != e->free_cells.end(); ++it)
        if (it->second >= need) break;
    if (it == e->free_cells.end()) return fail(OBGC_ERR_BUSY, "device budget exhausted");
    const int64_t off = it->first;
    const int64_t len = it->second;
    e->free_cells.erase(it);
    if (len > need) e->free_cells[off + need] = len - need;
    const int s = e->free_slots.back();
    e->free_slots.pop_back();
    ColSlot<double>& c = e->slots[s];
    std::memset(&c, 0, sizeof(c));
    c.cell_off = off; c.Nz = sp->Nz; c.steps_left = sp->nsteps; c.steps_done = 0;
    c.pulse_step = sp->pulse_step; c.pulse_k = sp->pulse_k; c.live = 1;
    c.dz = sp->dz; c.dt = sp->dt; c.PAR0 = sp->surface_PAR; c.mu0 = sp->mu0; c.pulse_amount = sp->pulse_amount;
    c.temp = sp->temperature; c.sal = sp->salinity;
    *slot = s;
    return OBGC_OK;
}

void release_column(obgc_columns* e, int64_t slot) {
    ColSlot<double>& c = e->slots[slot];
    int64_t off = c.cell_off, len = c.Nz + 1;
    c.live = 0;
    // return the block to the free list, merging neighbours
    auto next = e->free_cells.lower_bound(off);
    if (next != e->free_cells.end() && next->first == off + len) { len += next->second; e->free_cells.erase(next); }
    auto prev = e->free_cells.lower_bound(off);
    if (prev != e->free_cells.begin()) {
        --prev;
        if (prev->first + prev->second == off) { off = prev->first; len += prev->second; e->free_cells.erase(prev); }
    }
    e->free_cells[off] = len;
    e->free_slots.push_back((int)slot);
}

}  // namespace cols
}  // namespace obgc

using namespace obgc::cols;

extern "C" int obgc_columns_create(const obgc_columns_desc* d, obgc_columns** out) {
    if (!d || !out || d->max_columns < 1 || d->arena_cells < 1 || d->precision < OBGC_PREC_F32 ||
        d->precision > OBGC_PREC_MIXED)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_columns_create: bad descriptor");
    *out = nullptr;
    const int V = variant_of(d->npd);
    if (V != V_NPZD && V != V_LOBSTER_C)
        return fail(OBGC_ERR_UNSUPPORTED, "obgc_columns_create: columns support NPZD and LOBSTER with carbonates");
    if (d->gas_exchange != 0 &&
        (d->gas_exchange != 1 || V != V_LOBSTER_C || d->gas.gas != OBGC_GAS_CO2 || d->gas.wind_field || d->gas.air_field ||
         !valid_gas(&d->gas)))
        return fail(OBGC_ERR_INVALID_ARGUMENT,
                    "obgc_columns_create: gas_exchange is CO2 on LOBSTER columns with a constant wind and air concentration");
    obgc_columns* e = new obgc_columns();
    e->desc = *d;
    e->V = V;
    e->NT = V == V_NPZD ? 5 : 9;
    e->prec = d->precision;
    e->ts = d->precision == OBGC_PREC_F32 ? 4 : 8;
    e->threads = d->threads > 0 ? d->threads : 256;
    e->cap = d->pack_cells > 0 ? d->pack_cells : (e->ts == 4 ? 1024 : 512);
    int32_t req[32];
    required_tracers(&d->npd, req);
    for (int q = 0; q < e->NT; q++) e->names[q] = req[q];
    // sinking: only the two window tracers may drift
    const int WA = V == V_NPZD ? 1 : 4, WB = V == V_NPZD ? 4 : 5;
    for (int q = 0; q < e->NT; q++) {
        double w0 = 0;
        if (drift_speed(&d->npd, e->names[q], &w0) && w0 != 0.0) {
            if (q == WA) e->w0A = w0;
            else if (q == WB) e->w0B = w0;
            else { delete e; return fail(OBGC_ERR_UNSUPPORTED, "obgc_columns_create: only two tracers may sink"); }
        }
    }
    if (d->negatives < OBGC_NEGATIVES_NONE || d->negatives > OBGC_NEGATIVES_ZERO ||
        negatives_spec(d->npd, d->negatives, e->NT, e->names, d->zero_exclude, d->invalid_fill_value, &e->neg) != OBGC_OK) {
        delete e;
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_columns_create: bad negatives mode");
    }
    if (e->cap < OBGC_COLUMN_MAX_LEVELS || e->cap % 32 != 0 || e->threads % 32 != 0 || e->threads < COL_MAXC || e->threads > 512 ||
        smem_for(e, e->cap) > 227 * 1024) {
        delete e;
        return fail(OBGC_ERR_INVALID_ARGUMENT,
                    "obgc_columns_create: pack_cells (multiple of 32) must hold a 512-level column and fit shared memory; "
                    "threads a multiple of 32 from 64 to 512");
    }
    int rc = OBGC_OK;
    auto chk = [&](cudaError_t err, const char* w) { if (rc == OBGC_OK && err != cudaSuccess) rc = cuda_fail(err, w); };
    chk(cudaMalloc(&e->state, e->ts * e->NT * (size_t)d->arena_cells), "cudaMalloc(column state)");
    chk(cudaMalloc(&e->kappa, e->ts * (size_t)d->arena_cells), "cudaMalloc(column kappa)");
    const size_t sb = e->ts == 4 ? sizeof(ColSlot<float>) : sizeof(ColSlot<double>);
    chk(cudaMalloc(&e->d_slots, sb * d->max_columns), "cudaMalloc(slots)");
    chk(cudaMalloc((void**)&e->d_pack_slots, sizeof(int32_t) * d->max_columns), "cudaMalloc(pack slots)");
    chk(cudaMalloc((void**)&e->d_packs, sizeof(ColPack) * d->max_columns), "cudaMalloc(packs)");
    for (int b = 0; b < 2; b++) {
        chk(cudaMallocHost(&e->h_slots[b], sb * d->max_columns), "cudaMallocHost(slots)");
        chk(cudaMallocHost((void**)&e->h_pack_slots[b], sizeof(int32_t) * d->max_columns), "cudaMallocHost(pack slots)");
        chk(cudaMallocHost((void**)&e->h_packs[b], sizeof(ColPack) * d->max_columns), "cudaMallocHost(packs)");
        chk(cudaEventCreateWithFlags(&e->tables_ev[b], cudaEventDisableTiming), "cudaEventCreate(column tables)");
    }
    if (rc != OBGC_OK) { obgc_columns_destroy(e); return rc; }
    e->slots.resize(d->max_columns);
    for (auto& s : e->slots) std::memset(&s, 0, sizeof(s));
    for (int s = d->max_columns - 1; s >= 0; s--) e->free_slots.push_back(s);
    e->free_cells[0] = d->arena_cells;
    *out = e;
    return OBGC_OK;
}

extern "C" int obgc_columns_destroy(obgc_columns* e) {
    if (!e) return OBGC_OK;
    if (e->pending) cudaStreamSynchronize(e->last_stream);
    if (e->graph) cudaGraphExecDestroy(e->graph);
    if (e->capture_stream) cudaStreamDestroy(e->capture_stream);
    cudaFree(e->state); cudaFree(e->kappa); cudaFree(e->d_slots); cudaFree(e->d_pack_slots); cudaFree(e->d_packs);
    for (int b = 0; b < 2; b++) {
        cudaFreeHost(e->h_slots[b]); cudaFreeHost(e->h_pack_slots[b]); cudaFreeHost(e->h_packs[b]);
        if (e->tables_ev[b]) cudaEventDestroy(e->tables_ev[b]);
    }
    delete e;
    return OBGC_OK;
}

extern "C" int obgc_columns_tracers(const obgc_columns* e, int32_t* names, int32_t cap) {
    if (!e || !names || cap < e->NT) return -OBGC_ERR_INVALID_ARGUMENT;
    for (int q = 0; q < e->NT; q++) names[q] = e->names[q];
    return e->NT;
}

extern "C" int obgc_columns_add(obgc_columns* e, const obgc_column_spec* sp, const double* init, const double* kappa,
                                int64_t* slot) {
    if (!e || !sp || !init || !kappa || !slot || sp->Nz < 1 || sp->Nz > OBGC_COLUMN_MAX_LEVELS || sp->nsteps < 0 ||
        !(sp->dz > 0) || !(sp->dt > 0))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_columns_add: bad column");
    int64_t s = -1;
    const int rs = reserve_column(e, sp, &s);
    if (rs != OBGC_OK) return rs;
    const int64_t off = e->slots[s].cell_off;
    // stage the column's state and diffusivities on the engine's stream, then wait for the copies
    const size_t n = (size_t)e->NT * sp->Nz;
    cudaStream_t st = e->last_stream;
    int rc = OBGC_OK;
    if (e->ts == 4) {
        std::vector<float> a(init, init + n), k(kappa, kappa + sp->Nz + 1);
        OBGC_CUDA(cudaMemcpyAsync(static_cast<float*>(e->state) + off * e->NT, a.data(), 4 * n, cudaMemcpyHostToDevice, st));
        OBGC_CUDA(cudaMemcpyAsync(static_cast<float*>(e->kappa) + off, k.data(), 4 * (sp->Nz + 1), cudaMemcpyHostToDevice, st));
        e->pending = true;
        rc = drain(e);
    } else {
        OBGC_CUDA(cudaMemcpyAsync(static_cast<double*>(e->state) + off * e->NT, init, 8 * n, cudaMemcpyHostToDevice, st));
        OBGC_CUDA(cudaMemcpyAsync(static_cast<double*>(e->kappa) + off, kappa, 8 * (sp->Nz + 1), cudaMemcpyHostToDevice, st));
        e->pending = true;
        rc = drain(e);
    }
    if (rc != OBGC_OK) return rc;
    *slot = s;
    return OBGC_OK;
}

extern "C" int obgc_columns_advance(obgc_columns* e, int32_t max_steps, void* stream) {
    if (!e || max_steps < 1) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_columns_advance: bad argument");
    return advance_with(e, max_steps, e->threads, e->cap, static_cast<cudaStream_t>(stream), true);
}

extern "C" int obgc_columns_run(obgc_columns* e, int32_t nsteps, int32_t K, int32_t use_graph, void* stream) {
    if (!e || nsteps < 1 || K < 1) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_columns_run: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int npacks = stage_tables(e, e->cap, st);
    if (npacks <= 0) return -npacks;
    int rc = prepare_launch(e, e->cap);
    if (rc != OBGC_OK) return rc;
    const int nl = (nsteps + K - 1) / K;
    if (!use_graph) {
        for (int l = 0; l < nl && rc == OBGC_OK; l++) rc = launch_any(e, npacks, std::min(K, nsteps - l * K), e->threads, e->cap, st);
        if (rc != OBGC_OK) return rc;
        account_steps(e, nsteps);
        return OBGC_OK;
    }
    // The kernels read the slot and pack tables from fixed device buffers, so one captured graph
    // serves every run with the same grid (packs) and launch sequence.
    const int64_t key[5] = {npacks, nsteps, K, e->threads, e->cap};
    if (!e->graph || std::memcmp(key, e->graph_key, sizeof(key)) != 0) {
        if (e->graph) { cudaGraphExecDestroy(e->graph); e->graph = nullptr; }
        if (!e->capture_stream) OBGC_CUDA(cudaStreamCreateWithFlags(&e->capture_stream, cudaStreamNonBlocking));
        OBGC_CUDA(cudaStreamBeginCapture(e->capture_stream, cudaStreamCaptureModeThreadLocal));
        for (int l = 0; l < nl && rc == OBGC_OK; l++)
            rc = launch_any(e, npacks, std::min(K, nsteps - l * K), e->threads, e->cap, e->capture_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t end = cudaStreamEndCapture(e->capture_stream, &g);
        if (rc != OBGC_OK) { if (g) cudaGraphDestroy(g); return rc; }
        if (end != cudaSuccess) return cuda_fail(end, "cudaStreamEndCapture(columns)");
        const cudaError_t inst = cudaGraphInstantiate(&e->graph, g, 0);
        cudaGraphDestroy(g);
        if (inst != cudaSuccess) { e->graph = nullptr; return cuda_fail(inst, "cudaGraphInstantiate(columns)"); }
        count_launches(-(int64_t)nl);   // captured, not run: counted when replayed
        std::memcpy(e->graph_key, key, sizeof(key));
    }
    OBGC_CUDA(cudaGraphLaunch(e->graph, st));
    count_launches(nl);
    account_steps(e, nsteps);
    return OBGC_OK;
}

extern "C" int obgc_columns_remaining(const obgc_columns* e, int64_t slot, int32_t* left) {
    if (!e || !left || slot < 0 || slot >= (int64_t)e->slots.size() || !e->slots[slot].live)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_columns_remaining: bad slot");
    *left = e->slots[slot].steps_left;
    return OBGC_OK;
}

extern "C" int obgc_columns_read(obgc_columns* e, int64_t slot, double* out) {
    if (!e || !out || slot < 0 || slot >= (int64_t)e->slots.size() || !e->slots[slot].live)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_columns_read: bad slot");
    const ColSlot<double>& c = e->slots[slot];
    const size_t n = (size_t)e->NT * c.Nz;
    cudaStream_t st = e->last_stream;
    if (e->ts == 4) {
        std::vector<float> a(n);
        OBGC_CUDA(cudaMemcpyAsync(a.data(), static_cast<float*>(e->state) + c.cell_off * e->NT, 4 * n, cudaMemcpyDeviceToHost, st));
        e->pending = true;
        const int rc = drain(e);
        if (rc != OBGC_OK) return rc;
        for (size_t q = 0; q < n; q++) out[q] = a[q];
    } else {
        OBGC_CUDA(cudaMemcpyAsync(out, static_cast<double*>(e->state) + c.cell_off * e->NT, 8 * n, cudaMemcpyDeviceToHost, st));
        e->pending = true;
        return drain(e);
    }
    return OBGC_OK;
}

extern "C" int obgc_columns_remove(obgc_columns* e, int64_t slot) {
    if (!e || slot < 0 || slot >= (int64_t)e->slots.size() || !e->slots[slot].live)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_columns_remove: bad slot");
    release_column(e, slot);
    return OBGC_OK;
}

// Scratch of the autotuner (a copy of the arena's state, two timing events), released on every
// return path.
struct TuneScratch {
    void* saved = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    ~TuneScratch() {
        if (saved) cudaFree(saved);
        if (a) cudaEventDestroy(a);
        if (b) cudaEventDestroy(b);
    }
};

extern "C" int obgc_columns_autotune(obgc_columns* e, int32_t steps, int32_t* threads, int32_t* pack_cells, void* stream) {
    if (!e || steps < 1) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_columns_autotune: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int rc0 = drain(e);
    if (rc0 != OBGC_OK) return rc0;
    const size_t bytes = e->ts * e->NT * (size_t)e->desc.arena_cells;
    TuneScratch x;
    OBGC_CUDA(cudaMalloc(&x.saved, bytes));
    OBGC_CUDA(cudaEventCreate(&x.a));
    OBGC_CUDA(cudaEventCreate(&x.b));
    OBGC_CUDA(cudaMemcpyAsync(x.saved, e->state, bytes, cudaMemcpyDeviceToDevice, st));
    // time `steps` steps of one (threads, pack cap) pair from the saved state (after a warm-up run)
    auto time_pair = [&](int th, int cap, float* ms) -> int {
        int rc = advance_with(e, steps, th, cap, st, false);
        if (rc != OBGC_OK) return rc;
        OBGC_CUDA(cudaMemcpyAsync(e->state, x.saved, bytes, cudaMemcpyDeviceToDevice, st));
        OBGC_CUDA(cudaEventRecord(x.a, st));
        rc = advance_with(e, steps, th, cap, st, false);
        if (rc != OBGC_OK) return rc;
        OBGC_CUDA(cudaEventRecord(x.b, st));
        OBGC_CUDA(cudaEventSynchronize(x.b));
        OBGC_CUDA(cudaEventElapsedTime(ms, x.a, x.b));
        OBGC_CUDA(cudaMemcpyAsync(e->state, x.saved, bytes, cudaMemcpyDeviceToDevice, st));
        return OBGC_OK;
    };
    auto usable = [&](int cap) { return cap >= OBGC_COLUMN_MAX_LEVELS && smem_for(e, cap) <= 227 * 1024; };
    float best = 1e30f;
    int bt = e->threads, bc = e->cap;
    auto consider = [&](int th, int cap) -> int {
        if (!usable(cap)) return OBGC_OK;
        float ms = 0;
        const int rc = time_pair(th, cap, &ms);
        if (rc == OBGC_OK && ms < best) { best = ms; bt = th; bc = cap; }
        return rc;
    };
    // the pack size at 256 threads, then the block size at the best pack size, then the pack sizes
    // next to the best at that block size
    const int caps[] = {256, 384, 512, 768, 1024, 1536, 2048, 3072, 4096};
    const int ths[] = {64, 128, 192, 256, 320, 384, 448, 512};
    const int ncaps = (int)(sizeof(caps) / sizeof(caps[0]));
    int rc = OBGC_OK;
    for (int cap : caps)
        if ((rc = consider(256, cap)) != OBGC_OK) return rc;
    const int cap1 = bc;
    for (int th : ths)
        if (th != 256 && (rc = consider(th, cap1)) != OBGC_OK) return rc;
    const int th1 = bt;
    for (int q = 0; q < ncaps; q++)
        if (caps[q] == cap1) {
            if (q > 0 && (rc = consider(th1, caps[q - 1])) != OBGC_OK) return rc;
            if (q + 1 < ncaps && (rc = consider(th1, caps[q + 1])) != OBGC_OK) return rc;
        }
    OBGC_CUDA(cudaStreamSynchronize(st));
    e->threads = bt;
    e->cap = bc;
    if (threads) *threads = bt;
    if (pack_cells) *pack_cells = bc;
    return OBGC_OK;
}
