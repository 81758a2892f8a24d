// step_kernel.cuh — the fused RK3 substep of the 3-D model (mode (ii)).
//
// One launch per RK3 substep does, for every cell and every advected tracer:
//   G = BGC(U, PAR) - div(u c) - div(w_drift c)          (Oceananigans tracer tendency kernel,
//                                                         with the reference's BGC functors)
//   U_out = U + dt * (gamma G + zeta G-)                  (rk3_substep!, BoxModel/timesteppers.jl:79-93)
// and computes TwoBand PAR on the fly (update_TwoBandPhotosyntheticallyActiveRadiation!,
// src/Light/2band.jl:1-33) from the same state, so PAR never touches HBM.
//
// Work decomposition: a block of 32 x BY threads owns a 32 x BY tile of columns and a segment of
// TZ levels, marching from the top of the segment down.  The chlorophyll integral above the
// segment is summed first (reading only P), then carried down level by level.  Vertical face
// fluxes are carried in registers (each face reconstructed once).  Horizontal face fluxes are
// reconstructed once per face into shared memory; the 32+1-st x face and BY+1-st y face of each
// row/column are computed by one warp per tracer, rotating the warp with the tracer index so the
// extra work is spread evenly.  Blocks loop over work items (persistent grid).
#pragma once
#include "light_device.cuh"
#include "npd_device.cuh"
#include "weno_device.cuh"

namespace obgc {

constexpr int STEP_BX = 32;
constexpr int STEP_BY = 8;
constexpr int MAX_NT = 12;

// Tracer slot order of the fused variants: the reference's required_biogeochemical_tracers order,
// then T and S when they are carried without a BGC tendency.
__host__ __device__ constexpr int n_bgc(int V) {
    return V == V_NPZD ? 5 : (V == V_LOBSTER ? 7 : (V == V_LOBSTER_C ? 9 : (V == V_LOBSTER_CO ? 10 : 8)));
}
__host__ __device__ constexpr int slot_name(int V, int s) {
    // NPZD: N P Z T D ; LOBSTER: NO3 NH4 P Z sPOM bPOM DOM [DIC Alk] [O2]
    return V == V_NPZD
               ? (s == 0 ? OBGC_N : s == 1 ? OBGC_P : s == 2 ? OBGC_Z : s == 3 ? OBGC_T : s == 4 ? OBGC_D : OBGC_S)
               : (s == 0 ? OBGC_NO3 : s == 1 ? OBGC_NH4 : s == 2 ? OBGC_P : s == 3 ? OBGC_Z : s == 4 ? OBGC_SPOM
                  : s == 5 ? OBGC_BPOM : s == 6 ? OBGC_DOM
                  : (V == V_LOBSTER ? (s == 7 ? OBGC_T : OBGC_S)
                  : V == V_LOBSTER_O ? (s == 7 ? OBGC_O2 : s == 8 ? OBGC_T : OBGC_S)
                  : (s == 7 ? OBGC_DIC : s == 8 ? OBGC_ALK
                  : (V == V_LOBSTER_CO ? (s == 9 ? OBGC_O2 : s == 10 ? OBGC_T : OBGC_S)
                                       : (s == 9 ? OBGC_T : OBGC_S)))));
}
__host__ __device__ constexpr int slot_of_P(int V) { return V == V_NPZD ? 1 : 2; }

template <typename TS, typename TC>
struct SubstepArgs {
    int Nx, Ny, Nz;
    int periodic_x, periodic_y, flat_x, flat_y;
    int64_t sj, sk;
    TC dx, dy, dz, Lz;
    int TZ, nseg, ntx, nty, n_items;
    const TS* in[MAX_NT];
    TS* out[MAX_NT];
    TC* G[MAX_NT];
    const TS* u;
    const TS* v;
    const TS* w;
    const TC* drift;          // [MAX_NT][Nz+1] (only slots with a bit in drift_mask are read)
    uint32_t drift_mask;
    NPDParamsT<TC> bgc;
    TwoBandT<TC> light;
    int surf_kind;
    TC surf_value;            // OBGC_SURFACE_PAR_CONSTANT value
    const TS* surf_field;     // OBGC_SURFACE_PAR_FIELD
    const double* d_time;     // step start time (device), OBGC_SURFACE_PAR_DEFAULT
    double c_stage, dt_d;
    TC dt, gamma, zeta;
    int first_stage, write_G;
};

template <typename TS, typename TC>
__device__ __forceinline__ TC ld(const TS* p, int64_t i) { return TC(__ldg(p + i)); }

// Upwind-biased flux U * c_face at face f (between cells f-1 and f) of a line of N cells.
template <typename TS, typename TC>
__device__ __forceinline__ TC face_flux(const TS* __restrict__ line, int64_t s, int N, bool periodic, int f, TC U) {
    if (U == TC(0)) return TC(0);
    const bool pos = U > TC(0);
    if (periodic) {
        int m[6];
#pragma unroll
        for (int q = 0; q < 6; q++) {
            int x = f - 3 + q;
            x = x < 0 ? x + N : (x >= N ? x - N : x);
            m[q] = x;
        }
        const TC c0 = ld<TS, TC>(line, m[0] * s), c1 = ld<TS, TC>(line, m[1] * s), c2 = ld<TS, TC>(line, m[2] * s);
        const TC c3 = ld<TS, TC>(line, m[3] * s), c4 = ld<TS, TC>(line, m[4] * s), c5 = ld<TS, TC>(line, m[5] * s);
        const TC r = pos ? weno5(c0, c1, c2, c3, c4) : weno5(c5, c4, c3, c2, c1);
        return U * r;
    }
    const int b = f < N - f ? f : N - f;
    TC r;
    if (b >= 3) {
        const TC c0 = ld<TS, TC>(line, (int64_t)(f - 3) * s), c1 = ld<TS, TC>(line, (int64_t)(f - 2) * s);
        const TC c2 = ld<TS, TC>(line, (int64_t)(f - 1) * s), c3 = ld<TS, TC>(line, (int64_t)f * s);
        const TC c4 = ld<TS, TC>(line, (int64_t)(f + 1) * s), c5 = ld<TS, TC>(line, (int64_t)(f + 2) * s);
        r = pos ? weno5(c0, c1, c2, c3, c4) : weno5(c5, c4, c3, c2, c1);
    } else if (b == 2) {
        const TC c1 = ld<TS, TC>(line, (int64_t)(f - 2) * s), c2 = ld<TS, TC>(line, (int64_t)(f - 1) * s);
        const TC c3 = ld<TS, TC>(line, (int64_t)f * s), c4 = ld<TS, TC>(line, (int64_t)(f + 1) * s);
        r = pos ? weno3(c1, c2, c3) : weno3(c4, c3, c2);
    } else if (b == 1) {
        r = pos ? ld<TS, TC>(line, (int64_t)(f - 1) * s) : ld<TS, TC>(line, (int64_t)f * s);
    } else {
        r = ld<TS, TC>(line, (int64_t)(f == 0 ? 0 : N - 1) * s);
    }
    return U * r;
}

// Model velocity normal to face f of a line (zero at Bounded walls).
template <typename TS, typename TC>
__device__ __forceinline__ TC face_velocity(const TS* __restrict__ vel, int64_t base, int64_t s, int N, bool periodic, int f) {
    if (!vel) return TC(0);
    if (periodic) return ld<TS, TC>(vel, base + (int64_t)(f >= N ? f - N : f) * s);
    if (f <= 0 || f >= N) return TC(0);
    return ld<TS, TC>(vel, base + (int64_t)f * s);
}

template <typename TC, int NT>
constexpr size_t substep_smem_bytes() {
    return sizeof(TC) * NT * (STEP_BY * (STEP_BX + 1) + (STEP_BY + 1) * STEP_BX);
}

template <int V, int NT, typename TS, typename TC>
__global__ void __launch_bounds__(STEP_BX * STEP_BY, sizeof(TC) == 4 ? 2 : 1) substep_kernel(const SubstepArgs<TS, TC> a) {
    constexpr int NB = n_bgc(V);
    constexpr int SP = slot_of_P(V);
    constexpr int NWARP = STEP_BX * STEP_BY / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TC (*fx)[STEP_BY][STEP_BX + 1] = reinterpret_cast<TC (*)[STEP_BY][STEP_BX + 1]>(smem_raw);
    TC (*fy)[STEP_BY + 1][STEP_BX] =
        reinterpret_cast<TC (*)[STEP_BY + 1][STEP_BX]>(smem_raw + sizeof(TC) * NT * STEP_BY * (STEP_BX + 1));

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = tx + STEP_BX * ty;
    const int warp = tid >> 5, lane = tid & 31;
    const bool periodic_x = a.periodic_x, periodic_y = a.periodic_y;

    TC PAR0;
    if (a.surf_kind == OBGC_SURFACE_PAR_DEFAULT) PAR0 = TC(default_surface_par(*a.d_time + a.c_stage * a.dt_d));
    else PAR0 = a.surf_value;

    for (int item = blockIdx.x; item < a.n_items; item += gridDim.x) {
        const int seg = item % a.nseg;                       // top segment first
        const int tile = item / a.nseg;
        const int ti = tile % a.ntx, tj = tile / a.ntx;
        const int i0 = ti * STEP_BX, j0 = tj * STEP_BY;
        const int k_top = a.Nz - 1 - seg * a.TZ;
        const int k_bot = max(0, k_top - a.TZ + 1);
        const int i = i0 + tx, j = j0 + ty;
        const bool active = i < a.Nx && j < a.Ny;
        const int ic = min(i, a.Nx - 1), jc = min(j, a.Ny - 1);
        const int64_t col = ic + (int64_t)jc * a.sj;
        const TC P0 = a.surf_kind == OBGC_SURFACE_PAR_FIELD ? TC(a.surf_field[ic + (int64_t)jc * a.Nx]) : PAR0;

        // chlorophyll integral of the cells above the segment
        TC Sr = TC(0), Sb = TC(0);
        for (int k = a.Nz - 1; k > k_top; --k) {
            TC fr, fb;
            twoband_terms(a.light, ld<TS, TC>(a.in[SP], col + (int64_t)k * a.sk), fr, fb);
            Sr += fr;
            Sb += fb;
        }

        // vertical flux through the face above the segment (k_top + 1)
        TC Fz_up[NT];
#pragma unroll
        for (int t = 0; t < NT; t++) {
            Fz_up[t] = TC(0);
            const bool drifts = (a.drift_mask >> t) & 1u;
            if (a.w || drifts) {
                const TS* line = a.in[t] + col;
                const int f = k_top + 1;
                if (a.w) Fz_up[t] += face_flux<TS, TC>(line, a.sk, a.Nz, false, f, face_velocity<TS, TC>(a.w, col, a.sk, a.Nz, false, f));
                if (drifts) Fz_up[t] += face_flux<TS, TC>(line, a.sk, a.Nz, false, f, a.drift[t * (a.Nz + 1) + f]);
            }
        }

        for (int k = k_top; k >= k_bot; --k) {
            const int64_t idx = col + (int64_t)k * a.sk;
            TC c[NT];
#pragma unroll
            for (int t = 0; t < NT; t++) c[t] = ld<TS, TC>(a.in[t], idx);

            // PAR at this cell (2band.jl:26-31)
            TC fr, fb;
            twoband_terms(a.light, c[SP], fr, fb);
            const TC z = -a.Lz + (TC(k) + TC(0.5)) * a.dz;
            const TC PAR = twoband_par(a.light, P0, z, a.dz, Sr, Sb, fr, fb);
            Sr += fr;
            Sb += fb;

            // horizontal face fluxes
            __syncthreads();
#pragma unroll
            for (int t = 0; t < NT; t++) {
                if (!a.flat_x) {
                    const int64_t rowb = (int64_t)jc * a.sj + (int64_t)k * a.sk;
                    const TS* line = a.in[t] + rowb;
                    {
                        const int f = i;   // left face of this cell
                        TC F = TC(0);
                        if (active || (i <= a.Nx && j < a.Ny)) {
                            const TC U = face_velocity<TS, TC>(a.u, rowb, 1, a.Nx, periodic_x, f);
                            F = face_flux<TS, TC>(line, 1, a.Nx, periodic_x, f, U);
                        }
                        fx[t][ty][tx] = F;
                    }
                    if (warp == (2 * t) % NWARP && lane < STEP_BY) {
                        const int r = lane, jr = j0 + r;
                        const int f = i0 + STEP_BX;
                        TC F = TC(0);
                        if (jr < a.Ny && f <= a.Nx) {
                            const int64_t rb = (int64_t)jr * a.sj + (int64_t)k * a.sk;
                            const TC U = face_velocity<TS, TC>(a.u, rb, 1, a.Nx, periodic_x, f);
                            F = face_flux<TS, TC>(a.in[t] + rb, 1, a.Nx, periodic_x, f, U);
                        }
                        fx[t][r][STEP_BX] = F;
                    }
                }
                if (!a.flat_y) {
                    const int64_t cb = ic + (int64_t)k * a.sk;
                    const TS* line = a.in[t] + cb;
                    {
                        const int f = j;   // south face of this cell
                        TC F = TC(0);
                        if (i < a.Nx && j <= a.Ny) {
                            const TC U = face_velocity<TS, TC>(a.v, cb, a.sj, a.Ny, periodic_y, f);
                            F = face_flux<TS, TC>(line, a.sj, a.Ny, periodic_y, f, U);
                        }
                        fy[t][ty][tx] = F;
                    }
                    if (warp == (2 * t + 1) % NWARP) {
                        const int ix = i0 + lane;
                        const int f = j0 + STEP_BY;
                        TC F = TC(0);
                        if (ix < a.Nx && f <= a.Ny) {
                            const int64_t cb2 = ix + (int64_t)k * a.sk;
                            const TC U = face_velocity<TS, TC>(a.v, cb2, a.sj, a.Ny, periodic_y, f);
                            F = face_flux<TS, TC>(a.in[t] + cb2, a.sj, a.Ny, periodic_y, f, U);
                        }
                        fy[t][STEP_BY][lane] = F;
                    }
                }
            }
            __syncthreads();

            // named values for the BGC functors
            TC vals[OBGC_NUM_NAMED], g[OBGC_NUM_NAMED];
#pragma unroll
            for (int n = 0; n < OBGC_NUM_NAMED; n++) { vals[n] = TC(0); g[n] = TC(0); }
#pragma unroll
            for (int s = 0; s < NB; s++) vals[slot_name(V, s)] = c[s];
            npd_tendencies<V, TC>(a.bgc, vals, PAR, g);

#pragma unroll
            for (int t = 0; t < NT; t++) {
                TC adv = TC(0);
                if (!a.flat_x) adv += (fx[t][ty][tx + 1] - fx[t][ty][tx]) / a.dx;
                if (!a.flat_y) adv += (fy[t][ty + 1][tx] - fy[t][ty][tx]) / a.dy;
                const bool drifts = (a.drift_mask >> t) & 1u;
                if (a.w || drifts) {
                    const TS* line = a.in[t] + col;
                    TC Fz = TC(0);
                    if (a.w) Fz += face_flux<TS, TC>(line, a.sk, a.Nz, false, k, face_velocity<TS, TC>(a.w, col, a.sk, a.Nz, false, k));
                    if (drifts) Fz += face_flux<TS, TC>(line, a.sk, a.Nz, false, k, a.drift[t * (a.Nz + 1) + k]);
                    adv += (Fz_up[t] - Fz) / a.dz;
                    Fz_up[t] = Fz;
                }
                const TC Gt = (t < NB ? g[slot_name(V, t)] : TC(0)) - adv;
                if (active) {
                    TC Un;
                    if (a.first_stage) {
                        Un = a.dt * a.gamma * Gt;
                    } else {
                        const TC Gm = a.G[t][idx];
                        Un = a.dt * (a.gamma * Gt + a.zeta * Gm);
                    }
                    // accumulate in the storage precision (FP64 for the mixed path)
                    a.out[t][idx] = TS(__ldg(a.in[t] + idx)) + TS(Un);
                    if (a.write_G) a.G[t][idx] = Gt;
                }
            }
        }
    }
}

}  // namespace obgc
