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
#include <cuda.h>
#include "light_device.cuh"
#include "negatives.cuh"
#include "npd_device.cuh"
#include "weno_device.cuh"
#include "weno_x2.cuh"

namespace obgc {

constexpr int STEP_BX = 32;
constexpr int STEP_BY = 8;
constexpr int MAX_NT = 26;
constexpr int MAX_TOP = 4;      // surface-flux slots per launch
constexpr int MAX_FRC = 4;      // forced slots per launch

// Tracer slot order of the fused variants: the reference's required_biogeochemical_tracers order,
// then T and S when they are carried without a BGC tendency.
__host__ __device__ constexpr int n_bgc(int V) {
    return V == V_EXTERNAL ? 24
         : V == V_NPZD ? 5 : (V == V_LOBSTER ? 7 : (V == V_LOBSTER_C ? 9 : (V == V_LOBSTER_CO ? 10 : 8)));
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
    int64_t sj, sk;           // layout of the input arrays in[] (and of w)
    int64_t vsj, vsk;         // layout of u and v
    int64_t osj, osk;         // layout of the output arrays out[]
    int64_t gsj, gsk;         // layout of the tendency arrays G[] (and ext, bgc_out, frc)
    // TMA-staged stages of the mixed path (FP64 state in out[], updated in place): pout[t] is the
    // padded FP32 copy of the stage's new state, with its periodic images in the halos when out_halo,
    // from which the next stage copies its tiles (NULL: none, the call's last stage); layout psj, psk
    TC* pout[MAX_NT];
    int64_t psj, psk;
    // out[] are padded arrays (x halo of TMA_HX, y halo of HALO cells): the update also writes each
    // value into the halo cells that hold its periodic image, so the next stage can stage whole
    // tiles of it with the tensor-memory accelerator
    int out_halo;
    int tma_layout;           // non-zero: a stage of the TMA-staged steps (the MODE 2 instantiation)
    // tensor maps of in[] (3-D, box TMA_TILE_W x TILE_H x 1) in global memory, or NULL: the tiles are
    // then staged by per-element cp.async.  A tile at (i0, j0, k) is the box at (i0 + tma_x0,
    // j0 + tma_y0, k): (0, 0) for the padded sets, (-4, -3) for the caller's arrays, whose tiles
    // on a periodic edge (that would need the wrap) are staged by cp.async
    const CUtensorMap* tmap;
    int tma_x0, tma_y0;
    // a call's first stage when tmap holds the caller's arrays' maps: the tiles that need the
    // periodic wrap are copied from padded set 1 through these maps instead (at (i0, j0)); NULL: none
    const CUtensorMap* tmap_wrap;
    TC dx, dy, dz, Lz, inv_dx, inv_dy, inv_dz;
    int TZ, nseg, ntx, nty, n_items;
    const TS* in[MAX_NT];
    TS* out[MAX_NT];
    TC* G[MAX_NT];
    const TC* ext[MAX_NT];    // V_EXTERNAL: the BGC tendency of slot t (t < n_ext; NULL: none)
    int n_ext;                // V_EXTERNAL: slots of this launch with an external tendency
    // surface fluxes (air-sea gas exchange): slot top_slot1[q] - 1 (none when 0, so zeroed arguments
    // carry no flux) loses top_flux[q][i + j Nx] / dz in its surface cell: the divergence of a flux
    // through the top face, positive out of the ocean
    int top_slot1[MAX_TOP];
    const double* top_flux[MAX_TOP];
    // forcing: slot frc_slot1[q] - 1 gains the rate frc[q][idx] while the stage time lies in
    // [frc_t0[q], frc_t1[q])
    int frc_slot1[MAX_FRC];
    const TS* frc[MAX_FRC];
    double frc_t0[MAX_FRC], frc_t1[MAX_FRC];
    // CarbonateSystem replicates: the cell's BGC tendencies of DIC and Alk, written for the
    // launches of the replicate tracers (NULL: not written)
    TC* bgc_out[2];
    // negative-tracer modifier (update_state!) on the cell's new values, fused into the update
    // (mode OBGC_NEGATIVES_NONE: off)
    NegativesSpec neg;
    // ScalarDiffusivity with explicit time stepping: horizontal kh / dx and kh / dy fold a diffusive
    // flux -kh dc/dx into every x / y face flux (zero at Bounded walls); vertical: kzz[f] = kappa_f /
    // dz^2 at the Nz + 1 faces (zero at the bottom and top walls), or NULL for none
    TC kh_dx, kh_dy;
    const TC* kzz;
    // InstantRemineralisation sediment (src/Models/Sediments/instant_remineralisation.jl): the
    // sinking fluxes of the slots in sed_sink_mask through the bottom face deposit F per column; a
    // fraction e = a + b (F / (k + F))^2 is buried in sed_storage[i + j Nx] (RK3, previous-stage
    // burial in sed_G), the rest returns to slot sed_recv1 - 1 in the bottom cell (0: no sediment)
    int sed_recv1;
    uint32_t sed_sink_mask;
    // SimpleMultiGSediment: slot bot_slot1[q] - 1 gains bot_flux[q][i + j Nx] / dz in its bottom cell
    // (the sediment's coupled tendency of NO3, NH4, O2; none when 0)
    int bot_slot1[3];
    const double* bot_flux[3];
    TC sed_a, sed_b, sed_k;
    TS* sed_storage;
    TC* sed_G;
    const TS* u;
    const TS* v;
    const TS* w;
    const TC* drift;          // [MAX_NT][Nz+1] (only slots with a bit in drift_mask are read)
    uint32_t drift_mask;
    NPDParamsT<TC> bgc;
    TwoBandT<TC> light;
    // the chlorophyll sums of TwoBand PAR above each segment: par_prefix[(2 (s - 1) + b) Nx Ny + i + j Nx]
    // for segment s >= 1 and band b (red 0, blue 1), written by par_prefix_kernel before the launch;
    // NULL: each work item sums the cells above its segment itself
    const TC* par_prefix;
    // the TMA-staged instantiation (MODE 2): the vertical face fluxes of the two window slots,
    // written by sink_flux_kernel before the launch: fz_pre[(q (Nz + 1) + f) Nx Ny + i + j Nx] for
    // face f of window q (0: window_a, 1: window_b)
    const TC* fz_pre;
    int surf_kind;
    TC surf_value;            // OBGC_SURFACE_PAR_CONSTANT value
    const TS* surf_field;     // OBGC_SURFACE_PAR_FIELD
    const double* d_time;     // step start time (device), OBGC_SURFACE_PAR_DEFAULT
    int* status;              // OBGC_FLAG_NAN is set here when a stored value is not finite (NULL: no check)
    double c_stage, dt_d;
    TC dt, gamma, zeta;
    int first_stage, write_G;
};

template <typename TS, typename TC>
__device__ __forceinline__ TC ld(const TS* p, int64_t i) { return TC(__ldg(p + i)); }
// The exponent field of an FP64 value in place (bits 20-30 of its high word): 0x7ff00000 for a NaN
// or an infinity.
__device__ __forceinline__ unsigned d_exponent_bits(double x) { return (unsigned)__double2hiint(x) & 0x7ff00000u; }

// Asynchronous global -> shared copy of one 4- or 8-byte element (cp.async, sm_80+): no register
// staging; completed by cp_async_wait_all() before the barrier that publishes the shared data.
template <typename E>
__device__ __forceinline__ void cp_async_elem(E* smem, const E* gmem) {
    static_assert(sizeof(E) == 4 || sizeof(E) == 8, "cp.async element of 4 or 8 bytes");
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if constexpr (sizeof(E) == 4) asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(gmem) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(gmem) : "memory");
}
// The same with the shared-space address given directly (constant offsets fold into the instruction).
__device__ __forceinline__ void cp_async4_at(unsigned smem_addr, const void* gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_addr), "l"(gmem) : "memory");
}
__device__ __forceinline__ void prefetch_l2(const void* gmem) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(gmem));
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

// WENO5 of the upwind stencil: the five values are selected by the velocity sign first, so lanes
// of a warp with opposite signs still run one reconstruction.
template <typename TC>
__device__ __forceinline__ TC weno5_upwind(bool pos, TC c0, TC c1, TC c2, TC c3, TC c4, TC c5) {
    return weno5(pos ? c0 : c5, pos ? c1 : c4, pos ? c2 : c3, pos ? c3 : c2, pos ? c4 : c1);
}

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
        return U * weno5_upwind(pos, c0, c1, c2, c3, c4, c5);
    }
    const int b = f < N - f ? f : N - f;
    TC r;
    if (b >= 3) {
        const TC c0 = ld<TS, TC>(line, (int64_t)(f - 3) * s), c1 = ld<TS, TC>(line, (int64_t)(f - 2) * s);
        const TC c2 = ld<TS, TC>(line, (int64_t)(f - 1) * s), c3 = ld<TS, TC>(line, (int64_t)f * s);
        const TC c4 = ld<TS, TC>(line, (int64_t)(f + 1) * s), c5 = ld<TS, TC>(line, (int64_t)(f + 2) * s);
        r = weno5_upwind(pos, c0, c1, c2, c3, c4, c5);
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

constexpr int HALO = 3;
// A tile holds TILE_H rows of the cells x = i0 - 3 .. i0 + 34 that the stencils of a 32 x 8 tile
// read (38 values).  With TMA staging a row holds x = i0 - 4 .. i0 + 35 (40 values), so that the
// tensor copy's box starts at x = i0 - 4, a multiple of 4 FP32 values (16 bytes), and x = i0 - 3 sits
// in column 1.
constexpr int TILE_H = STEP_BY + 2 * HALO;
constexpr int TILE_CELLS = (STEP_BX + 2 * HALO) * TILE_H;   // the cells a tile stages
constexpr int TILE_LOADS = (TILE_CELLS + STEP_BX * STEP_BY - 1) / (STEP_BX * STEP_BY);
constexpr int TMA_TILE_W = STEP_BX + 8;
constexpr int TMA_HX = 4;                                   // x halo of the padded arrays

// Whether the tile at (i0, j0) needs the periodic wrap: its staged halo leaves the grid in a
// periodic direction.
__host__ __device__ inline bool tile_wraps_xy(int i0, int j0, int Nx, int Ny, bool periodic_x, bool periodic_y) {
    return (periodic_x && (i0 < TMA_HX || i0 + TMA_TILE_W - TMA_HX > Nx)) || (periodic_y && (j0 < HALO || j0 + STEP_BY + HALO > Ny));
}
template <typename TS, typename TC>
__host__ __device__ inline bool tile_wraps(const SubstepArgs<TS, TC>& a, int i0, int j0) {
    return tile_wraps_xy(i0, j0, a.Nx, a.Ny, a.periodic_x, a.periodic_y);
}
template <bool SPLIT>
__host__ __device__ constexpr int tile_w() { return SPLIT ? TMA_TILE_W : STEP_BX + 2 * HALO; }
template <bool SPLIT>
__host__ __device__ constexpr int tile_x0() { return SPLIT ? 1 : 0; }
// shared-memory elements per tracer tile: in the TMA-staged instantiations rounded up to 128 bytes
// (the alignment of a tensor copy's destination)
template <typename TC, bool SPLIT>
__host__ __device__ constexpr int tile_elems() {
    return SPLIT ? ((TMA_TILE_W * TILE_H * (int)sizeof(TC) + 127) / 128) * 128 / (int)sizeof(TC) : TILE_CELLS;
}

template <typename TC, int NT, bool SPLIT = false>
constexpr size_t substep_smem_bytes() {
    // every tracer's tile (first: 128-byte aligned), the fx, fy face fluxes, and the carried
    // vertical flux and its divergence
    return sizeof(TC) * NT * (tile_elems<TC, SPLIT>() + STEP_BY * (STEP_BX + 1) + (STEP_BY + 1) * STEP_BX + 2 * STEP_BX * STEP_BY);
}

// The two slots whose vertical stencil the kernel keeps in register windows (LOBSTER: sPOM, bPOM;
// NPZD: P, D; PISCES' middle launch: POC, GOC).
__host__ __device__ constexpr int window_a(int V) { return V == V_NPZD ? 1 : V == V_EXTERNAL ? 1 : 4; }
__host__ __device__ constexpr int window_b(int V) { return V == V_NPZD ? 4 : V == V_EXTERNAL ? 2 : 5; }

// ---- tensor-memory-accelerator staging: one mbarrier per block, armed by thread 0 with the bytes
// of every tracer's tile of a level, completed by the tile copies
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arm(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    unsigned done;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done) : "r"(smem_u32(bar)), "r"(parity) : "memory");
    return done != 0;
}
// Box (TMA_TILE_W x TILE_H x 1) of a padded array at padded coordinates (x, y, z) into shared memory.
__device__ __forceinline__ void tma_tile(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar)) : "memory");
}
// A wait on the staging mbarrier gives up after this many polls (each poll may suspend the thread
// for a while): the block then goes on with whatever the tile holds and reports OBGC_FLAG_TIMEOUT.
constexpr unsigned TMA_MAX_POLLS = 1u << 22;

// Face flux from six tile values s[0], s[st], ..., s[5 st] = c[f-3 .. f+2] of a line of N cells,
// with the Bounded-wall order reduction of face_flux.
template <typename TC>
__device__ __forceinline__ TC tile_face_flux(const TC* s, int st, bool periodic, int f, int N, TC U) {
    if (U == TC(0)) return TC(0);
    const bool pos = U > TC(0);
    const int b = periodic ? 3 : min(f, N - f);
    TC r;
    if (b >= 3) r = weno5_upwind(pos, s[0], s[st], s[2 * st], s[3 * st], s[4 * st], s[5 * st]);
    else if (b == 2) r = pos ? weno3(s[st], s[2 * st], s[3 * st]) : weno3(s[4 * st], s[3 * st], s[2 * st]);
    else if (b == 1) r = pos ? s[2 * st] : s[3 * st];
    else r = TC(0);
    return U * r;
}

// Diffusive flux -coef (c[f] - c[f-1]) through face f of a line of N cells (s as in tile_face_flux:
// s[2 st] = c[f-1], s[3 st] = c[f]); zero at the walls of a bounded line.
template <typename TC>
__device__ __forceinline__ TC tile_diff_flux(const TC* s, int st, bool periodic, int f, int N, TC coef) {
    if (coef == TC(0) || (!periodic && (f <= 0 || f >= N))) return TC(0);
    return -coef * (s[3 * st] - s[2 * st]);
}

// Vertical face flux from a window w0..w5 = c[f-3 .. f+2] (same order reduction and wall rule as
// face_flux: a wall face takes the adjacent interior value).
template <typename TC>
__device__ __forceinline__ TC window_face_flux(TC w0, TC w1, TC w2, TC w3, TC w4, TC w5, int f, int N, TC U) {
    if (U == TC(0)) return TC(0);
    const bool pos = U > TC(0);
    const int b = min(f, N - f);
    TC r;
    if (b >= 3) r = weno5_upwind(pos, w0, w1, w2, w3, w4, w5);
    else if (b == 2) r = pos ? weno3(w1, w2, w3) : weno3(w4, w3, w2);
    else if (b == 1) r = pos ? w2 : w3;
    else r = f == 0 ? w3 : w2;
    return U * r;
}

__device__ __forceinline__ int wrap_or_clamp(int x, int N, bool periodic) {
    if (periodic) {
        while (x < 0) x += N;
        while (x >= N) x -= N;
        return x;
    }
    return min(max(x, 0), N - 1);
}

// Flux of tracer line `line` through vertical face f: advective (model w and the tracer's drift
// velocity, when `adv`) plus the explicit vertical diffusion -kappa_f dc/dz (none at the walls).
template <typename TS, typename TC>
__device__ __forceinline__ TC vertical_flux(const SubstepArgs<TS, TC>& a, const TS* __restrict__ line, int64_t col,
                                            int t, int f, bool adv = true) {
    TC F = TC(0);
    if (adv && a.w) F += face_flux<TS, TC>(line, a.sk, a.Nz, false, f, face_velocity<TS, TC>(a.w, col, a.sk, a.Nz, false, f));
    if (adv && ((a.drift_mask >> t) & 1u)) F += face_flux<TS, TC>(line, a.sk, a.Nz, false, f, a.drift[t * (a.Nz + 1) + f]);
    if (a.kzz && f > 0 && f < a.Nz)
        F -= a.kzz[f] * a.dz * (ld<TS, TC>(line, (int64_t)f * a.sk) - ld<TS, TC>(line, (int64_t)(f - 1) * a.sk));
    return F;
}

// Whether a launch uses any of the optional terms (diffusivity closure, surface fluxes, forcing,
// the fused negative-tracer modifier, the sediment, replicate tendencies); without them the lean
// instantiation (EXT = false) runs.
template <typename TS, typename TC>
__host__ __device__ inline bool substep_needs_ext(const SubstepArgs<TS, TC>& a) {
    bool any = a.kh_dx != TC(0) || a.kh_dy != TC(0) || a.kzz != nullptr || a.neg.mode != OBGC_NEGATIVES_NONE ||
               a.sed_recv1 != 0 || a.bgc_out[0] != nullptr || a.bgc_out[1] != nullptr;
    for (int q = 0; q < 3; q++) any = any || a.bot_slot1[q] != 0;
    for (int q = 0; q < MAX_TOP; q++) any = any || a.top_slot1[q] != 0;
    for (int q = 0; q < MAX_FRC; q++) any = any || a.frc_slot1[q] != 0;
    return any;
}

// MODE 0: every array in the input layout, tiles staged by cp.async.  MODE 2: the TMA-staged steps'
// instantiation: input, output and tendency arrays in their own layouts (a.sj/sk, osj/osk, gsj/gsk;
// u and v in vsj/vsk), 40-wide tile rows, every tile copied by tensor copies through a.tmap (from a
// padded set, or from the caller's arrays when none of their tiles needs the periodic wrap), and
// periodic halo images written when a.out_halo is set (mixed precision: out[] is the FP64 state,
// updated in place, and the FP32 padded copy pout[] takes the images).
template <int V, int NT, typename TS, typename TC, bool EXT, int MODE = 0>
__global__ void __launch_bounds__(STEP_BX * STEP_BY, sizeof(TC) != 4 ? 1 : NT <= 12 ? 3 : NT <= 16 ? 2 : 1)
    substep_kernel(const __grid_constant__ SubstepArgs<TS, TC> a) {
    constexpr bool SPLIT = MODE != 0;
    constexpr bool TMA = MODE == 2;
    // mixed precision with TMA-staged tiles: the FP64 state is updated in place (a thread reads and
    // writes only its own cells of it) and the tiles come from the FP32 padded copies (pout)
    constexpr bool MIX2 = TMA && sizeof(TS) != sizeof(TC);
    constexpr int TILE_W = tile_w<SPLIT>();
    constexpr int TILE_X0 = tile_x0<SPLIT>();
    constexpr int NB = n_bgc(V);
    constexpr int SP = slot_of_P(V);
    constexpr int NTH = STEP_BX * STEP_BY;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    constexpr int TILE_SZ = tile_elems<TC, SPLIT>();
    TC* tiles = reinterpret_cast<TC*>(smem_raw);     // NT tiles of TILE_H rows of TILE_W
    unsigned char* after_tiles = smem_raw + sizeof(TC) * NT * TILE_SZ;
    TC (*fx)[STEP_BY][STEP_BX + 1] = reinterpret_cast<TC (*)[STEP_BY][STEP_BX + 1]>(after_tiles);
    TC (*fy)[STEP_BY + 1][STEP_BX] =
        reinterpret_cast<TC (*)[STEP_BY + 1][STEP_BX]>(after_tiles + sizeof(TC) * NT * STEP_BY * (STEP_BX + 1));
    TC* fzu = reinterpret_cast<TC*>(after_tiles + sizeof(TC) * NT * (STEP_BY * (STEP_BX + 1) + (STEP_BY + 1) * STEP_BX));
    TC* vdv = fzu + NT * NTH;
    __shared__ uint64_t stage_bar;   // TMA staging (MODE 2)

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = tx + STEP_BX * ty;
    const bool periodic_x = a.periodic_x, periodic_y = a.periodic_y;
    // Sinking tracers advance their vertical stencil in a register window (one new load per
    // level); two window slots per variant (LOBSTER: sPOM, bPOM; NPZD: P, D).  Any other
    // vertically advected tracer, and every tracer when a model w is given, takes the generic path.
    // PISCES (V_EXTERNAL, launched on tracers 0-8, 9-17 and 18-25): POC and GOC are slots 1 and 2
    // of the second launch; the other four sinking tracers take the generic path.
    constexpr int WA = window_a(V), WB = window_b(V);
    // MODE 2 reads the window slots' face fluxes from sink_flux_kernel instead (no window
    // registers: they were 12 % of a launch)
    constexpr bool PREFZ = MODE != 0;
    const bool winA = !PREFZ && a.w == nullptr && ((a.drift_mask >> WA) & 1u);
    const bool winB = !PREFZ && a.w == nullptr && ((a.drift_mask >> WB) & 1u);
    const bool preA = PREFZ && ((a.drift_mask >> WA) & 1u);
    const bool preB = PREFZ && ((a.drift_mask >> WB) & 1u);
    // tracers whose vertical advection takes the generic path, and those whose vertical face flux
    // does (the generic advection set, plus every tracer under explicit vertical diffusion)
    const uint32_t adv_mask = a.w != nullptr ? 0xffffffffu : (a.drift_mask & ~((1u << WA) | (1u << WB)));
    const uint32_t gen_mask = (EXT && a.kzz != nullptr) ? 0xffffffffu : adv_mask;
    const bool any_generic = (gen_mask & ((1u << NT) - 1u)) != 0u;
    // explicit horizontal diffusivity (rare: off in the common configurations)
    const bool hdiff = EXT && (a.kh_dx != TC(0) || a.kh_dy != TC(0));
    // previous-stage tendencies staged in shared memory (the generic-drift buffer, when unused)
    const bool gm_smem = !any_generic && !a.first_stage;
    // shared-space address of the tiles
    const unsigned tiles_s = smem_u32(tiles);
    unsigned tma_phase = 0;
    bool tma_timeout = false;
    if (TMA) {
        // a tensor copy's destination must be 128-byte aligned: never issue one to a tile that is not
        // (the block then does no work and reports OBGC_FLAG_TIMEOUT)
        if ((tiles_s & 127u) != 0u) {
            if (tid == 0 && a.status) atomicOr(a.status, OBGC_FLAG_TIMEOUT);
            return;
        }
        if (tid == 0) mbar_init(&stage_bar, 1);
        __syncthreads();
    }
    (void)tma_phase;
    constexpr unsigned TILE_BYTES = (unsigned)(sizeof(TC) * TMA_TILE_W * TILE_H);
    // thread 0 arms the barrier and copies every tracer's tile of level kk of the work item at
    // (i0, j0): the box whose first cell is x = i0 - 4, y = j0 - 3 of the grid
    auto tma_issue = [&](int i0_, int j0_, int kk) {
        const bool wrap = a.tmap_wrap != nullptr && tile_wraps(a, i0_, j0_);
        const CUtensorMap* maps = wrap ? a.tmap_wrap : a.tmap;
        const int x0 = i0_ + (wrap ? 0 : a.tma_x0), y0 = j0_ + (wrap ? 0 : a.tma_y0);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arm(&stage_bar, TILE_BYTES * NT);
#pragma unroll 1
        for (int t = 0; t < NT; t++) tma_tile(tiles + t * TILE_SZ, maps + t, x0, y0, kk, &stage_bar);
    };

    // forcings switched on at this stage's time
    bool frc_on[MAX_FRC];
#pragma unroll
    for (int q = 0; q < MAX_FRC; q++) frc_on[q] = false;
    if constexpr (EXT) {
        bool any_frc = false;
#pragma unroll
        for (int q = 0; q < MAX_FRC; q++) any_frc = any_frc || a.frc_slot1[q] != 0;
        if (any_frc) {   // d_time is only required of launches with a forcing
            const double t_stage = *a.d_time + a.c_stage * a.dt_d;
#pragma unroll
            for (int q = 0; q < MAX_FRC; q++)
                frc_on[q] = a.frc_slot1[q] != 0 && t_stage >= a.frc_t0[q] && t_stage < a.frc_t1[q];
        }
    }

    TC PAR0 = TC(0);
    if constexpr (V != V_EXTERNAL) {
        if (a.surf_kind == OBGC_SURFACE_PAR_DEFAULT) PAR0 = TC(default_surface_par(*a.d_time + a.c_stage * a.dt_d));
        else PAR0 = a.surf_value;
    }

    bool bad = false;   // a non-finite value was stored by this thread
    // FP32: NaN-or-infinity detector on the FMA pipe, fma(U, 0, acc) (0 for a finite U, NaN otherwise),
    // in place of a compare and a predicate OR per stored value on the busier ALU pipe
    TS nanacc = TS(0);
    // FP64: the largest exponent field stored, on the integer pipe (all ones: a NaN or an infinity)
    // in place of an FP64 compare per value on GB300's narrow FP64 pipe
    unsigned expmax = 0u;
    for (int item = blockIdx.x; item < a.n_items; item += gridDim.x) {
        const int seg = item % a.nseg;                       // top segment first
        const int tile = item / a.nseg;
        const int ti = tile % a.ntx, tj = tile / a.ntx;
        const int i0 = ti * STEP_BX, j0 = tj * STEP_BY;
        const int k_top = a.Nz - 1 - seg * a.TZ;
        const int k_bot = max(0, k_top - a.TZ + 1);
        const int i = i0 + tx, j = j0 + ty;
        const bool active = i < a.Nx && j < a.Ny;
        // tile rows past the grid (a 2-D grid with Flat y uses one of the eight) skip the arithmetic
        // (warp-uniform: a warp is one row); the row just past the last cell row still owns the y
        // faces of the tile's northern edge
        const bool row_cells = j < a.Ny;
        const bool row_faces = row_cells || (j == a.Ny && !a.flat_y);
        const int ic = min(i, a.Nx - 1), jc = min(j, a.Ny - 1);
        const int64_t col = ic + (int64_t)jc * a.sj;
        const TC P0 = (V != V_EXTERNAL && a.surf_kind == OBGC_SURFACE_PAR_FIELD) ? TC(a.surf_field[ic + (int64_t)jc * a.Nx])
                                                                                 : PAR0;

        // horizontal offsets of the tile elements this thread stages (the same for every level
        // and tracer of the work item)
        // tensor copies in MODE 2 (a Bounded direction's out-of-range cells are filled with zeros,
        // which only the unused stencil cells beyond a wall read)
        constexpr bool item_tma = TMA;
        int64_t toff[TILE_LOADS];
#pragma unroll
        for (int q = 0; q < (TMA ? 0 : TILE_LOADS); q++) {
            const int e = min(tid + q * NTH, TILE_CELLS - 1);
            const int r = e / (STEP_BX + 2 * HALO), c = e - r * (STEP_BX + 2 * HALO);
            toff[q] = wrap_or_clamp(i0 - HALO + c, a.Nx, periodic_x) +
                      (int64_t)wrap_or_clamp(j0 - HALO + r, a.Ny, periodic_y) * a.sj;
        }
        // shared-memory element of staged cell q (dense rows, or 40-wide rows with x = i0 - 3 in
        // column 1 in the TMA-staged instantiations)
        auto soff = [&](int q) -> int {
            const int e = tid + q * NTH;
            return SPLIT ? e + (TILE_W - (STEP_BX + 2 * HALO)) * (e / (STEP_BX + 2 * HALO)) + TILE_X0 : e;
        };

        // chlorophyll integral of the cells above the segment: from the pre-pass, or summed here
        TC Sr = TC(0), Sb = TC(0);
        if constexpr (V != V_EXTERNAL) {
            if (a.par_prefix != nullptr) {
                if (seg > 0) {
                    const int64_t cols = (int64_t)a.Nx * a.Ny, c2 = ic + (int64_t)jc * a.Nx;
                    Sr = a.par_prefix[(int64_t)(2 * seg - 2) * cols + c2];
                    Sb = a.par_prefix[(int64_t)(2 * seg - 1) * cols + c2];
                }
            } else {
#pragma unroll 1
                for (int k = a.Nz - 1; k > k_top; --k) {
                    TC fr, fb;
                    twoband_terms(a.light, ld<TS, TC>(a.in[SP], col + (int64_t)k * a.sk), fr, fb);
                    Sr += fr;
                    Sb += fb;
                }
            }
        }

        // vertical flux through the face above the segment (k_top + 1), carried per thread in smem
        if (any_generic) {
#pragma unroll 1
            for (int t = 0; t < NT; t++) {
                const bool vert = (gen_mask >> t) & 1u;
                fzu[t * NTH + tid] = vert ? vertical_flux(a, a.in[t] + col, col, t, k_top + 1, (adv_mask >> t) & 1u) : TC(0);
                vdv[t * NTH + tid] = TC(0);
            }
        }
        // register windows wA/wB = c[k-3 .. k+3] of the two window tracers, and their carried
        // flux through the face above the current level
        TC wA[7], wB[7], FzA = TC(0), FzB = TC(0);
#pragma unroll
        for (int m = 0; m < 7; m++) {
            const int kk = min(max(k_top - 3 + m, 0), a.Nz - 1);
            wA[m] = winA ? ld<TS, TC>(a.in[WA], col + (int64_t)kk * a.sk) : TC(0);
            wB[m] = winB ? ld<TS, TC>(a.in[WB], col + (int64_t)kk * a.sk) : TC(0);
        }
        if (winA) FzA = window_face_flux(wA[1], wA[2], wA[3], wA[4], wA[5], wA[6], k_top + 1, a.Nz, a.drift[WA * (a.Nz + 1) + k_top + 1]);
        if (winB) FzB = window_face_flux(wB[1], wB[2], wB[3], wB[4], wB[5], wB[6], k_top + 1, a.Nz, a.drift[WB * (a.Nz + 1) + k_top + 1]);
        const int64_t fz_cols = (int64_t)a.Nx * a.Ny, fz_c = ic + (int64_t)jc * a.Nx;
        if (preA) FzA = a.fz_pre[(int64_t)(k_top + 1) * fz_cols + fz_c];
        if (preB) FzB = a.fz_pre[(int64_t)(a.Nz + 1 + k_top + 1) * fz_cols + fz_c];

#pragma unroll 1
        for (int k = k_top; k >= k_bot; --k) {
            const int64_t idx = col + (int64_t)k * a.sk;                                      // in[]
            const int64_t gidx = SPLIT ? ic + (int64_t)jc * a.gsj + (int64_t)k * a.gsk : idx;   // G[], EXT fields
            const int64_t kofs = (int64_t)k * a.sk;
            // stage every tracer's tile and halo for this level: all loads in flight together (FP32:
            // asynchronous copies, no registers), and, from the second stage on, the cell's previous
            // tendencies into the generic-drift buffer when no tracer uses it
            if (item_tma) {
                // the tiles of this level: issued here at the item's first level, otherwise during
                // the previous level's update
                if (tid == 0 && k == k_top) tma_issue(i0, j0, k);
                // the previous tendencies into this thread's own slots: waited for just before the
                // update reads them, so the loads fly during the face loop
#pragma unroll 1
                for (int t = 0; t < NT; t++)
                    if (gm_smem) cp_async_elem<TC>(vdv + t * NTH + tid, a.G[t] + gidx);
                // mixed: this cell's FP64 values, read again by the update, into L2 meanwhile
                if constexpr (MIX2) {
#pragma unroll 1
                    for (int t = 0; t < NT; t++) prefetch_l2(a.in[t] + idx);
                }
                unsigned polls = 0;
                if (!tma_timeout)
                    while (!mbar_try_wait(&stage_bar, tma_phase & 1u))
                        if (++polls >= TMA_MAX_POLLS) { tma_timeout = true; break; }
                tma_phase++;
            } else {
#pragma unroll
                for (int t = 0; t < NT; t++) {
                    const TS* __restrict__ base = a.in[t] + kofs;
                    TC* tl = tiles + t * TILE_SZ;
#pragma unroll
                    for (int q = 0; q < TILE_LOADS; q++)
                        if (q < TILE_LOADS - 1 || tid + q * NTH < TILE_CELLS) {
                            if constexpr (sizeof(TS) == 4 && sizeof(TC) == 4)
                                cp_async4_at(tiles_s + 4u * (unsigned)(t * TILE_SZ + soff(q)), base + toff[q]);
                            else tl[soff(q)] = ld<TS, TC>(base, toff[q]);
                        }
                    if (gm_smem) cp_async_elem<TC>(vdv + t * NTH + tid, a.G[t] + gidx);
                }
                if constexpr (sizeof(TS) == 4 && sizeof(TC) == 4) cp_async_wait_all();
                else if (gm_smem) cp_async_wait_all();
            }
            const int64_t vsj = SPLIT ? a.vsj : a.sj;
            const int64_t vk = (int64_t)k * (SPLIT ? a.vsk : a.sk);
            const int64_t rowb = (int64_t)jc * vsj + vk;
            const int64_t cb = ic + vk;
            const bool xok = !a.flat_x && i <= a.Nx && j < a.Ny;
            const bool yok = !a.flat_y && i < a.Nx && j <= a.Ny;
            const TC Ux = xok ? face_velocity<TS, TC>(a.u, rowb, 1, a.Nx, periodic_x, i) : TC(0);
            const TC Uy = yok ? face_velocity<TS, TC>(a.v, cb, vsj, a.Ny, periodic_y, j) : TC(0);
            const bool full5 = (periodic_x || min(i, a.Nx - i) >= 3) && (periodic_y || min(j, a.Ny - j) >= 3);
            __syncthreads();

            // west (x) and south (y) faces of this thread's cell for every tracer: one (not
            // unrolled) loop keeps the code inside the instruction cache; in FP32 the two
            // reconstructions run as one packed f32x2 WENO5
#pragma unroll 1
            for (int t = 0; t < (row_faces ? NT : 0); t++) {
                const TC* tl = tiles + t * TILE_SZ;
                const TC* xs = tl + (ty + HALO) * TILE_W + TILE_X0 + tx;   // c[i-3 .. i+2] along x
                const TC* ys = tl + ty * TILE_W + TILE_X0 + tx + HALO;     // c[j-3 .. j+2] along y
                TC Fx, Fy;
#ifdef __CUDA_ARCH__
                if constexpr (sizeof(TC) == 4) {
                    if (full5) {
                        const bool pxp = Ux > TC(0), pyp = Uy > TC(0);
                        const f32x2 r = weno5_x2(
                            pk2(pxp ? xs[0] : xs[5], pyp ? ys[0] : ys[5 * TILE_W]),
                            pk2(pxp ? xs[1] : xs[4], pyp ? ys[TILE_W] : ys[4 * TILE_W]),
                            pk2(pxp ? xs[2] : xs[3], pyp ? ys[2 * TILE_W] : ys[3 * TILE_W]),
                            pk2(pxp ? xs[3] : xs[2], pyp ? ys[3 * TILE_W] : ys[2 * TILE_W]),
                            pk2(pxp ? xs[4] : xs[1], pyp ? ys[4 * TILE_W] : ys[TILE_W]));
                        float rx, ry;
                        up2(r, rx, ry);
                        Fx = Ux == TC(0) ? TC(0) : Ux * rx;
                        Fy = Uy == TC(0) ? TC(0) : Uy * ry;
                    } else {
                        Fx = tile_face_flux<TC>(xs, 1, periodic_x, i, a.Nx, Ux);
                        Fy = tile_face_flux<TC>(ys, TILE_W, periodic_y, j, a.Ny, Uy);
                    }
                } else
#endif
                {
                    Fx = tile_face_flux<TC>(xs, 1, periodic_x, i, a.Nx, Ux);
                    Fy = tile_face_flux<TC>(ys, TILE_W, periodic_y, j, a.Ny, Uy);
                }
                fx[t][ty][tx] = Fx;
                fy[t][ty][tx] = Fy;
                if ((gen_mask >> t) & 1u) {
                    const TC Fz = vertical_flux(a, a.in[t] + col, col, t, k, (adv_mask >> t) & 1u);   // face below this cell
                    vdv[t * NTH + tid] = (fzu[t * NTH + tid] - Fz) * a.inv_dz;
                    fzu[t * NTH + tid] = Fz;
                }
            }
            // explicit horizontal diffusion: -kappa dc/dx and -kappa dc/dy added to this thread's faces
            if (hdiff && row_faces) {
#pragma unroll 1
                for (int t = 0; t < NT; t++) {
                    const TC* tl = tiles + t * TILE_SZ;
                    if (xok) fx[t][ty][tx] += tile_diff_flux<TC>(tl + (ty + HALO) * TILE_W + TILE_X0 + tx, 1, periodic_x, i, a.Nx, a.kh_dx);
                    if (yok) fy[t][ty][tx] += tile_diff_flux<TC>(tl + ty * TILE_W + TILE_X0 + tx + HALO, TILE_W, periodic_y, j, a.Ny, a.kh_dy);
                }
            }
            // the tile's east (8 per tracer) and north (32 per tracer) edge faces, spread over
            // every thread of the block
            constexpr int NEDGE = STEP_BY + STEP_BX;
            bool edges_done = false;
#ifdef __CUDA_ARCH__
            if constexpr (sizeof(TC) == 4) {
                // FP32 without horizontal diffusion: the 40 edge faces of a tracer as 20 pairs, each one
                // packed WENO5 (east face r with north face r for r < 8, then the remaining north faces
                // two by two), so one pass over the block covers up to 12 tracers; a pair with a face
                // next to a wall takes the scalar reconstruction of each face
                if (!hdiff) {
                    constexpr int NPAIR = NEDGE / 2;
                    // face q of a pair: its stencil (6 values c[f-3 .. f+2], stride st), face index f of
                    // a line of N cells, periodicity, and its normal velocity (0 where it has no flux)
                    auto edge_face = [&](int t, int e, const TC*& s, int& st, int& f, int& N, bool& per, TC& U) {
                        const TC* tl = tiles + t * TILE_SZ;
                        if (e < STEP_BY) {
                            const int jr = j0 + e;
                            f = i0 + STEP_BX; N = a.Nx; per = periodic_x; st = 1;
                            s = tl + (e + HALO) * TILE_W + TILE_X0 + STEP_BX;
                            U = (!a.flat_x && jr < a.Ny && f <= a.Nx)
                                    ? face_velocity<TS, TC>(a.u, (int64_t)jr * vsj + vk, 1, a.Nx, periodic_x, f) : TC(0);
                        } else {
                            const int cc = e - STEP_BY, ix = i0 + cc;
                            f = j0 + STEP_BY; N = a.Ny; per = periodic_y; st = TILE_W;
                            s = tl + STEP_BY * TILE_W + TILE_X0 + cc + HALO;
                            U = (!a.flat_y && ix < a.Nx && f <= a.Ny)
                                    ? face_velocity<TS, TC>(a.v, ix + vk, vsj, a.Ny, periodic_y, f) : TC(0);
                        }
                    };
                    auto store_face = [&](int t, int e, TC F) {
                        if (e < STEP_BY) fx[t][e][STEP_BX] = F;
                        else fy[t][STEP_BY][e - STEP_BY] = F;
                    };
#pragma unroll 1
                    for (int p = tid; p < NT * NPAIR; p += NTH) {
                        const int t = p / NPAIR, r = p - t * NPAIR;
                        const int eA = r < STEP_BY ? r : STEP_BY + 2 * r - STEP_BY;      // 0..7, then north 8, 10, ..
                        const int eB = r < STEP_BY ? STEP_BY + r : eA + 1;               // north 0..7, then 9, 11, ..
                        const TC *sA, *sB;
                        int stA, stB, fA, fB, NA, NB;
                        bool perA, perB;
                        TC UA, UB;
                        edge_face(t, eA, sA, stA, fA, NA, perA, UA);
                        edge_face(t, eB, sB, stB, fB, NB, perB, UB);
                        if ((perA || min(fA, NA - fA) >= 3) && (perB || min(fB, NB - fB) >= 3)) {
                            const bool pa = UA > TC(0), pb = UB > TC(0);
                            const f32x2 w = weno5_x2(pk2(pa ? sA[0] : sA[5 * stA], pb ? sB[0] : sB[5 * stB]),
                                                     pk2(pa ? sA[stA] : sA[4 * stA], pb ? sB[stB] : sB[4 * stB]),
                                                     pk2(pa ? sA[2 * stA] : sA[3 * stA], pb ? sB[2 * stB] : sB[3 * stB]),
                                                     pk2(pa ? sA[3 * stA] : sA[2 * stA], pb ? sB[3 * stB] : sB[2 * stB]),
                                                     pk2(pa ? sA[4 * stA] : sA[stA], pb ? sB[4 * stB] : sB[stB]));
                            float ra, rb;
                            up2(w, ra, rb);
                            store_face(t, eA, UA == TC(0) ? TC(0) : UA * ra);
                            store_face(t, eB, UB == TC(0) ? TC(0) : UB * rb);
                        } else {
                            store_face(t, eA, tile_face_flux<TC>(sA, stA, perA, fA, NA, UA));
                            store_face(t, eB, tile_face_flux<TC>(sB, stB, perB, fB, NB, UB));
                        }
                    }
                    edges_done = true;
                }
            }
#endif
#pragma unroll 1
            for (int e = edges_done ? NT * NEDGE : tid; e < NT * NEDGE; e += NTH) {
                const int t = e / NEDGE, r = e - t * NEDGE;
                const TC* tl = tiles + t * TILE_SZ;
                if (r < STEP_BY) {
                    const int jr = j0 + r, f = i0 + STEP_BX;
                    TC Fe = TC(0);
                    if (!a.flat_x && jr < a.Ny && f <= a.Nx) {
                        const int64_t rb = (int64_t)jr * vsj + vk;
                        Fe = tile_face_flux<TC>(tl + (r + HALO) * TILE_W + TILE_X0 + STEP_BX, 1, periodic_x, f, a.Nx,
                                                face_velocity<TS, TC>(a.u, rb, 1, a.Nx, periodic_x, f));
                        if (hdiff) Fe += tile_diff_flux<TC>(tl + (r + HALO) * TILE_W + TILE_X0 + STEP_BX, 1, periodic_x, f, a.Nx, a.kh_dx);
                    }
                    fx[t][r][STEP_BX] = Fe;
                } else {
                    const int cc = r - STEP_BY, ix = i0 + cc, f = j0 + STEP_BY;
                    TC Fe = TC(0);
                    if (!a.flat_y && ix < a.Nx && f <= a.Ny) {
                        const int64_t cb2 = ix + vk;
                        Fe = tile_face_flux<TC>(tl + STEP_BY * TILE_W + TILE_X0 + cc + HALO, TILE_W, periodic_y, f, a.Ny,
                                                face_velocity<TS, TC>(a.v, cb2, vsj, a.Ny, periodic_y, f));
                        if (hdiff) Fe += tile_diff_flux<TC>(tl + STEP_BY * TILE_W + TILE_X0 + cc + HALO, TILE_W, periodic_y, f, a.Ny, a.kh_dy);
                    }
                    fy[t][STEP_BY][cc] = Fe;
                }
            }
            // this cell's value of every tracer: read after the face loop (not live across it) and
            // before the barrier that lets the next level's staging overwrite the tiles
            TC c[NT];
#pragma unroll
            for (int t = 0; t < NT; t++) c[t] = tiles[t * TILE_SZ + (ty + HALO) * TILE_W + TILE_X0 + tx + HALO];
            __syncthreads();
            // the tiles are free again: the next level's copies fly during this level's update
            if (item_tma && tid == 0 && k > k_bot) tma_issue(i0, j0, k - 1);
            if (TMA && gm_smem) cp_async_wait_all();   // this thread's previous tendencies (every thread)
            if (!row_cells) continue;   // no cell on this row: nothing below reads its registers

            // window tracers: flux through the face below this cell, divergence, and slide the
            // windows down one level (the next level needs c[k-4])
            TC vdA = TC(0), vdB = TC(0);
            bool win_done = false;
#ifdef __CUDA_ARCH__
            if constexpr (sizeof(TC) == 4) {
                // both windows at an interior face: one packed f32x2 WENO5 (the same arithmetic per
                // element as the scalar path below)
                const TC UA = winA ? a.drift[WA * (a.Nz + 1) + k] : TC(0), UB = winB ? a.drift[WB * (a.Nz + 1) + k] : TC(0);
                if (UA != TC(0) && UB != TC(0) && min(k, a.Nz - k) >= 3) {
                    const bool pa = UA > TC(0), pb = UB > TC(0);
                    const f32x2 r = weno5_x2(pk2(pa ? wA[0] : wA[5], pb ? wB[0] : wB[5]), pk2(pa ? wA[1] : wA[4], pb ? wB[1] : wB[4]),
                                             pk2(pa ? wA[2] : wA[3], pb ? wB[2] : wB[3]), pk2(pa ? wA[3] : wA[2], pb ? wB[3] : wB[2]),
                                             pk2(pa ? wA[4] : wA[1], pb ? wB[4] : wB[1]));
                    float ra, rb;
                    up2(r, ra, rb);
                    const TC FA = UA * ra, FB = UB * rb;
                    vdA = (FzA - FA) * a.inv_dz;
                    FzA = FA;
                    vdB = (FzB - FB) * a.inv_dz;
                    FzB = FB;
                    win_done = true;
                }
            }
#endif
            if (!win_done && winA) {
                const TC F = window_face_flux(wA[0], wA[1], wA[2], wA[3], wA[4], wA[5], k, a.Nz, a.drift[WA * (a.Nz + 1) + k]);
                vdA = (FzA - F) * a.inv_dz;
                FzA = F;
            }
            if (!win_done && winB) {
                const TC F = window_face_flux(wB[0], wB[1], wB[2], wB[3], wB[4], wB[5], k, a.Nz, a.drift[WB * (a.Nz + 1) + k]);
                vdB = (FzB - F) * a.inv_dz;
                FzB = F;
            }
            if (preA) {
                const TC F = a.fz_pre[(int64_t)k * fz_cols + fz_c];
                vdA = (FzA - F) * a.inv_dz;
                FzA = F;
            }
            if (preB) {
                const TC F = a.fz_pre[(int64_t)(a.Nz + 1 + k) * fz_cols + fz_c];
                vdB = (FzB - F) * a.inv_dz;
                FzB = F;
            }
            // the sediment: deposition through the bottom face, its burial and the remineralised rest
            TC sed_remin = TC(0);
            if constexpr (EXT) {
                if (a.sed_recv1 != 0 && k == 0) {
                    TC dep = TC(0);
#pragma unroll 1
                    for (int t = 0; t < NT; t++) {
                        if (!((a.sed_sink_mask >> t) & 1u)) continue;
                        const TC Fb = t == WA && winA ? FzA : t == WB && winB ? FzB
                                    : ((gen_mask >> t) & 1u) ? fzu[t * NTH + tid] : TC(0);
                        dep -= Fb;   // downward (negative) flux deposits
                    }
                    const TC r = dep / (a.sed_k + dep);
                    const TC e = a.sed_a + a.sed_b * (r * r);
                    sed_remin = (TC(1) - e) * dep * a.inv_dz;
                    if (active) {
                        const int64_t c2 = ic + (int64_t)jc * a.Nx;
                        const TC burial = e * dep;
                        const TC upd = a.first_stage ? a.dt * a.gamma * burial
                                                     : a.dt * (a.gamma * burial + a.zeta * a.sed_G[c2]);
                        a.sed_storage[c2] += TS(upd);
                        if (a.write_G) a.sed_G[c2] = burial;
                    }
                }
            }
            if (k > k_bot) {
                const int64_t nk = col + (int64_t)max(k - 4, 0) * a.sk;
#pragma unroll
                for (int m = 6; m > 0; m--) { wA[m] = wA[m - 1]; wB[m] = wB[m - 1]; }
                if (winA) wA[0] = ld<TS, TC>(a.in[WA], nk);
                if (winB) wB[0] = ld<TS, TC>(a.in[WB], nk);
            }

            TC g[V == V_EXTERNAL ? 1 : OBGC_NUM_NAMED];
            if constexpr (V != V_EXTERNAL) {
                // PAR at this cell (2band.jl:26-31)
                TC fr, fb;
                twoband_terms(a.light, c[SP], fr, fb);
                const TC z = -a.Lz + (TC(k) + TC(0.5)) * a.dz;
                const TC PAR = twoband_par(a.light, P0, z, a.dz, Sr, Sb, fr, fb);
                Sr += fr;
                Sb += fb;

                // named values for the BGC functors
                TC vals[OBGC_NUM_NAMED];
#pragma unroll
                for (int n = 0; n < OBGC_NUM_NAMED; n++) { vals[n] = TC(0); g[n] = TC(0); }
#pragma unroll
                for (int s = 0; s < NB; s++) vals[slot_name(V, s)] = c[s];
                npd_tendencies<V, TC>(a.bgc, vals, PAR, g);
                if constexpr (EXT) {
                    if (active && a.bgc_out[0]) a.bgc_out[0][gidx] = g[OBGC_DIC];
                    if (active && a.bgc_out[1]) a.bgc_out[1][gidx] = g[OBGC_ALK];
                }
            }

            const int64_t oidx = SPLIT ? ic + (int64_t)jc * a.osj + (int64_t)k * a.osk : idx;   // out[]
            // the periodic images of this cell in a padded output's halo: x = i -/+ Nx for the first
            // and last TMA_HX columns, y = j -/+ Ny for the first and last HALO rows (none: 0)
            int img_x = 0, img_y = 0;
            if (SPLIT && a.out_halo) {
                if (periodic_x) img_x = i < TMA_HX ? a.Nx : (i >= a.Nx - TMA_HX ? -a.Nx : 0);
                const int ysj = (int)(MIX2 ? a.psj : a.osj);
                if (periodic_y) img_y = j < HALO ? a.Ny * ysj : (j >= a.Ny - HALO ? -a.Ny * ysj : 0);
            }
#pragma unroll
            for (int t = 0; t < NT; t++) {
                TC adv = TC(0);
                if (!a.flat_x) adv += (fx[t][ty][tx + 1] - fx[t][ty][tx]) * a.inv_dx;
                if (!a.flat_y) adv += (fy[t][ty + 1][tx] - fy[t][ty][tx]) * a.inv_dy;
                if (any_generic) adv += vdv[t * NTH + tid];
                if (t == WA) adv += vdA;
                if (t == WB) adv += vdB;
                TC Gb = TC(0);
                if constexpr (V == V_EXTERNAL) {
                    if (t < a.n_ext && a.ext[t] != nullptr) Gb = a.ext[t][gidx];
                } else {
                    if (t < NB) Gb = g[slot_name(V, t)];
                }
                TC Gt = Gb - adv;
                if constexpr (EXT) {
                    if (t + 1 == a.sed_recv1) Gt += sed_remin;   // zero above the bottom cell
                    if (k == 0) {
#pragma unroll
                        for (int q = 0; q < 3; q++)
                            if (t + 1 == a.bot_slot1[q]) Gt += TC(a.bot_flux[q][ic + (int64_t)jc * a.Nx]) * a.inv_dz;
                    }
                    if (k == a.Nz - 1) {
#pragma unroll
                        for (int q = 0; q < MAX_TOP; q++)
                            if (t + 1 == a.top_slot1[q]) Gt -= TC(a.top_flux[q][ic + (int64_t)jc * a.Nx]) * a.inv_dz;
                    }
#pragma unroll
                    for (int q = 0; q < MAX_FRC; q++)
                        if (frc_on[q] && t + 1 == a.frc_slot1[q] && active) Gt += ld<TS, TC>(a.frc[q], gidx);
                }
                if (active) {
                    TC Un;
                    if (a.first_stage) {
                        Un = a.dt * a.gamma * Gt;
                    } else {
                        const TC Gm = gm_smem ? vdv[t * NTH + tid] : a.G[t][gidx];
                        Un = a.dt * (a.gamma * Gt + a.zeta * Gm);
                    }
                    // accumulate in the storage precision (FP64 for the mixed path)
                    TS Uo;
                    if constexpr (sizeof(TS) == sizeof(TC)) Uo = c[t] + Un;
                    else if constexpr (MIX2) Uo = a.in[t][idx] + TS(Un);   // in place: a plain load
                    else Uo = TS(__ldg(a.in[t] + idx)) + TS(Un);
                    a.out[t][oidx] = Uo;
                    if constexpr (sizeof(TS) == 4) nanacc = fmaf(Uo, 0.f, nanacc);
                    else expmax = max(expmax, d_exponent_bits(Uo));
                    if constexpr (MIX2) {
                        if (a.pout[t]) {
                            const int64_t pidx = ic + (int64_t)jc * a.psj + (int64_t)k * a.psk;
                            const TC Up = TC(Uo);   // the rounding the cp.async staging applies
                            a.pout[t][pidx] = Up;
                            if (img_x) a.pout[t][pidx + img_x] = Up;
                            if (img_y) a.pout[t][pidx + img_y] = Up;
                        }
                    } else if (SPLIT) {
                        if (img_x) a.out[t][oidx + img_x] = Uo;
                        if (img_y) a.out[t][oidx + img_y] = Uo;
                    }
                    if (a.write_G) a.G[t][gidx] = Gt;
                }
            }
            // ScaleNegativeTracers / ZeroNegativeTracers on the values this thread just stored,
            // the update_state! that follows the substep (negative_tracers.jl:136-276)
            if constexpr (EXT) {
                if (a.neg.mode != OBGC_NEGATIVES_NONE && active) {
                    negatives_cell<TS>(a.neg, [&](int q) -> TS& { return a.out[q][oidx]; });
#pragma unroll 1
                    for (int t = 0; t < NT; t++) bad |= !(fabs(a.out[t][oidx]) <= TS(INFINITY));
                }
            }
        }
    }
    bad |= !(nanacc == TS(0)) || expmax == 0x7ff00000u;
    if (bad && a.status) atomicOr(a.status, OBGC_FLAG_NAN);
    if (tma_timeout && a.status) atomicOr(a.status, OBGC_FLAG_TIMEOUT);
}

// The vertical face fluxes of the two window slots (the sinking tracers) at every face of every
// column, for the TMA-staged substep launch that follows (its fz_pre).  A block takes 32 columns;
// each of its warps takes SF_FACES consecutive faces, loading the SF_FACES + 5 levels their stencils
// span once (clamped to the grid, as the substep's windows are).  A face's two fluxes are formed
// exactly as the windows form them: one packed WENO5 where both drift speeds are non-zero at an
// interior face, window_face_flux otherwise (the same arithmetic per element, so the fluxes are bit
// for bit the windows').
constexpr int SF_FACES = 4;   // faces a thread: four ran faster than eight or sixteen
template <typename TS, typename TC>
__global__ void __launch_bounds__(256) sink_flux_kernel(const TS* __restrict__ cA, const TS* __restrict__ cB, int64_t sj,
                                                        int64_t sk, int Nx, int Ny, int Nz, const TC* __restrict__ drift,
                                                        int WA, int WB, TC* __restrict__ out) {
    const int64_t cols = (int64_t)Nx * Ny;
    const int64_t c = (int64_t)blockIdx.x * 32 + threadIdx.x % 32;
    const int f0 = (blockIdx.y * 8 + threadIdx.x / 32) * SF_FACES;   // this thread's first face
    if (c >= cols || f0 > Nz) return;
    const int64_t col = (c % Nx) + (c / Nx) * sj;
    TC wA[SF_FACES + 5], wB[SF_FACES + 5];   // c[f0 - 3 .. f0 + SF_FACES + 1]
#pragma unroll
    for (int m = 0; m < SF_FACES + 5; m++) {
        const int64_t kk = min(max(f0 - 3 + m, 0), Nz - 1);
        wA[m] = ld<TS, TC>(cA, col + kk * sk);
        wB[m] = ld<TS, TC>(cB, col + kk * sk);
    }
#pragma unroll
    for (int q = 0; q < SF_FACES; q++) {
        const int f = f0 + q;
        if (f > Nz) break;
        const TC UA = drift[WA * (Nz + 1) + f], UB = drift[WB * (Nz + 1) + f];
        TC FA, FB;
        bool done = false;
#ifdef __CUDA_ARCH__
        if constexpr (sizeof(TC) == 4) {
            if (UA != TC(0) && UB != TC(0) && min(f, Nz - f) >= 3) {
                const bool pa = UA > TC(0), pb = UB > TC(0);
                const f32x2 r = weno5_x2(pk2(pa ? wA[q] : wA[q + 5], pb ? wB[q] : wB[q + 5]),
                                         pk2(pa ? wA[q + 1] : wA[q + 4], pb ? wB[q + 1] : wB[q + 4]),
                                         pk2(pa ? wA[q + 2] : wA[q + 3], pb ? wB[q + 2] : wB[q + 3]),
                                         pk2(pa ? wA[q + 3] : wA[q + 2], pb ? wB[q + 3] : wB[q + 2]),
                                         pk2(pa ? wA[q + 4] : wA[q + 1], pb ? wB[q + 4] : wB[q + 1]));
                float ra, rb;
                up2(r, ra, rb);
                FA = UA * ra;
                FB = UB * rb;
                done = true;
            }
        }
#endif
        if (!done) {
            FA = window_face_flux(wA[q], wA[q + 1], wA[q + 2], wA[q + 3], wA[q + 4], wA[q + 5], f, Nz, UA);
            FB = window_face_flux(wB[q], wB[q + 1], wB[q + 2], wB[q + 3], wB[q + 4], wB[q + 5], f, Nz, UB);
        }
        out[(int64_t)f * cols + c] = FA;
        out[(int64_t)(Nz + 1 + f) * cols + c] = FB;
    }
}

// The chlorophyll sums of TwoBand PAR above the top of every segment of TZ levels but the first,
// for the substep launch that follows (its par_prefix).  A block takes PP_COLS columns: its eight
// warps evaluate the terms of PP_CHUNK levels at a time into shared memory (all loads and powers of
// a chunk in parallel), then the first warp adds them up per column from the surface down, in the
// order the substep kernel's own loop does (the same terms and additions, so the sums are bit for
// bit the ones a work item would form), and writes the sum at each segment's top.  Each work item of
// the substep then reads two values instead of summing up to Nz - TZ levels.
constexpr int PP_COLS = 32;
constexpr int PP_CHUNK = 64;
template <typename TS, typename TC>
__global__ void __launch_bounds__(256) par_prefix_kernel(const TS* __restrict__ P, int64_t sj, int64_t sk, int Nx, int Ny,
                                                         int Nz, int TZ, int nseg, TwoBandT<TC> L, TC* __restrict__ out) {
    __shared__ TC fr_s[PP_CHUNK][PP_COLS], fb_s[PP_CHUNK][PP_COLS];
    const int64_t cols = (int64_t)Nx * Ny;
    const int col = threadIdx.x % PP_COLS, lane = threadIdx.x / PP_COLS;   // lane: 0 .. 7
    const int64_t c = (int64_t)blockIdx.x * PP_COLS + col;
    const bool live = c < cols;
    const TS* p = P + (live ? (c % Nx) + (c / Nx) * sj : 0);
    const int nlev = (nseg - 1) * TZ;   // the levels above the last segment's top, from the surface
    TC Sr = TC(0), Sb = TC(0);
    int s = 1;                          // the next segment whose sum is due
    for (int c0 = 0; c0 < nlev; c0 += PP_CHUNK) {
        const int n = min(PP_CHUNK, nlev - c0);
        // this thread's levels of the chunk: every load in flight first, then the terms
        constexpr int PER = PP_CHUNK / (256 / PP_COLS);
        TC v[PER];
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int q = lane + u * (256 / PP_COLS);
            v[u] = live && q < n ? ld<TS, TC>(p, (int64_t)(Nz - 1 - (c0 + q)) * sk) : TC(0);
        }
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int q = lane + u * (256 / PP_COLS);
            if (q < n) {
                TC fr = TC(0), fb = TC(0);
                if (live) twoband_terms(L, v[u], fr, fb);
                fr_s[q][col] = fr;
                fb_s[q][col] = fb;
            }
        }
        __syncthreads();
        if (lane == 0) {
            for (int q = 0; q < n; q++) {
                Sr += fr_s[q][col];
                Sb += fb_s[q][col];
                if (c0 + q + 1 == s * TZ) {   // the levels above segment s are summed
                    if (live) {
                        out[(int64_t)(2 * s - 2) * cols + c] = Sr;
                        out[(int64_t)(2 * s - 1) * cols + c] = Sb;
                    }
                    s++;
                }
            }
        }
        __syncthreads();
    }
}

}  // namespace obgc
