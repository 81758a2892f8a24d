// pisces_model.cu — a 3-D PISCES model stepped on the device.
//
// Per RK3 stage (the order of Oceananigans' update_state! followed by the tendency kernels):
//   negative-tracer modifier (optional) -> chlorophyll PChl + DChl -> MultiBand PAR bands and their
//   sum -> euphotic depth -> mixed-layer PAR -> calcite saturation (FP64, warm-started) ->
//   all 24 PISCES tendencies (pisces_kernel) -> one fused substep: WENO5 advection of the 26
//   tracers, sinking, RK3 update (substep_kernel<V_EXTERNAL, 26>).
// The sinking speeds are built once, as the reference's setup_velocity_fields does at construction:
// POC at a constant speed, GOC by DepthDependantSinkingSpeed with the prescribed mixed-layer depth
// and the euphotic depth the model starts with (zero), so every column shares one profile.
#include <cmath>
#include <cstring>
#include <vector>
#include "negatives.cuh"
#include "pisces_device.cuh"
#include "step_launch.cuh"

extern "C" int obgc_multiband_par(int32_t nbands, const double* kw, const double* e, const double* chi, const double* division,
                                  const obgc_surface* surface, const obgc_grid* grid, int32_t dtype, const void* Chl,
                                  void* const* band_fields, void* PAR_total, double t, void* stream);
extern "C" int obgc_euphotic_depth(const obgc_surface* surface, const obgc_grid* grid, int32_t dtype, const void* PAR,
                                   void* zeu, double cutoff, double t, void* stream);
extern "C" int obgc_mixed_layer_mean(const obgc_grid* grid, int32_t dtype, const void* field,
                                     const obgc_pisces_field* mixed_layer_depth, void* out, void* stream);

namespace obgc {

int multiband_par_mixed(int nb, const double* kw, const double* e, const double* chi, const double* dv,
                        const obgc_surface* s, const obgc_grid* g, const void* Chl, void* const* bands, void* total,
                        double t, cudaStream_t st);

template <typename TS, typename T>
int launch_pisces(const obgc_pisces_params* p, const obgc_grid* g, const void* const* tracers, const obgc_pisces_field* aux,
                  void* const* G, double t, cudaStream_t st);
template <typename T>
int launch_pisces_omega(const obgc_carbon_options* opt, const obgc_grid* grid, const void* DIC, const void* Alk,
                        const void* Tc, const void* S, const void* Si, void* Omega, double* H_inout, int* fails,
                        cudaStream_t st);

namespace {

constexpr int PNT = OBGC_PIS_NUM;

template <typename T>
__global__ void chl_sum_kernel(const T* PChl, const T* DChl, T* Chl, int Nx, int Ny, int Nz, int64_t sj, int64_t sk) {
    const int64_t N = (int64_t)Nx * Ny * Nz;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % Nx);
        const int64_t r = c / Nx;
        const int64_t o = i + (r % Ny) * sj + (r / Ny) * sk;
        Chl[o] = PChl[o] + DChl[o];
    }
}

template <typename T>
struct CopyFields {
    const T* src[PNT];
    T* dst[PNT];
};

template <typename T>
__global__ void copy_fields_kernel(const __grid_constant__ CopyFields<T> F, int Nx, int Ny, int Nz, int64_t sj, int64_t sk) {
    const int64_t N = (int64_t)Nx * Ny * Nz;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % Nx);
        const int64_t r = c / Nx;
        const int64_t o = i + (r % Ny) * sj + (r / Ny) * sk;
#pragma unroll 1
        for (int q = 0; q < PNT; q++) F.dst[q][o] = F.src[q][o];
    }
}

// conserved_tracers(::PISCES) (coupling_utils.jl:11-33) as a negatives spec over the PISCES slots.
NegativesSpec pisces_negatives_spec(const obgc_pisces_params& p, double fill) {
    NegativesSpec s;
    std::memset(&s, 0, sizeof(s));
    s.mode = OBGC_NEGATIVES_SCALE;
    s.nt = PNT;
    s.fill = fill;
    auto group = [&](std::initializer_list<int> slots, std::initializer_list<double> f) {
        const int g = s.ng++;
        int m = 0;
        auto fi = f.begin();
        for (int q : slots) { s.slot[g][m] = q; s.fac[g][m] = *fi++; m++; }
        s.gn[g] = m;
    };
    const double tP = p.phosphate_redfield_ratio, tN = p.nitrogen_redfield_ratio;
    group({OBGC_PIS_P, OBGC_PIS_D, OBGC_PIS_Z, OBGC_PIS_M, OBGC_PIS_DOC, OBGC_PIS_POC, OBGC_PIS_GOC, OBGC_PIS_DIC, OBGC_PIS_CACO3},
          {1, 1, 1, 1, 1, 1, 1, 1, 1});
    group({OBGC_PIS_PFE, OBGC_PIS_DFE, OBGC_PIS_Z, OBGC_PIS_M, OBGC_PIS_SFE, OBGC_PIS_BFE, OBGC_PIS_FE},
          {1, 1, p.micro.iron_ratio, p.meso.iron_ratio, 1, 1, 1});
    group({OBGC_PIS_P, OBGC_PIS_D, OBGC_PIS_Z, OBGC_PIS_M, OBGC_PIS_DOC, OBGC_PIS_POC, OBGC_PIS_GOC, OBGC_PIS_PO4},
          {tP, tP, tP, tP, tP, tP, tP, 1});
    group({OBGC_PIS_DSI, OBGC_PIS_SI, OBGC_PIS_PSI}, {1, 1, 1});
    group({OBGC_PIS_NH4, OBGC_PIS_NO3, OBGC_PIS_P, OBGC_PIS_D, OBGC_PIS_Z, OBGC_PIS_M, OBGC_PIS_DOC, OBGC_PIS_POC, OBGC_PIS_GOC},
          {1, 1, tN, tN, tN, tN, tN, tN, tN});
    return s;
}

}  // namespace
}  // namespace obgc

using namespace obgc;

struct obgc_pisces_model {
    obgc_pisces_model_desc desc;
    size_t ts = 4, tc = 4;
    int64_t extent = 0;                  // elements spanned by a centre field (stride_k * Nz)
    void* user[PNT] = {};
    void* scratch[PNT] = {};
    void* G[PNT] = {};                   // previous-stage total tendencies (compute precision)
    void* Gb[OBGC_PIS_NUM_BGC] = {};     // biogeochemical tendencies of the stage
    void* chl = nullptr;
    void* par[4] = {};                   // total, bands 1..3
    void* zeu = nullptr;                 // (Nx, Ny)
    void* mlpar = nullptr;               // (Nx, Ny)
    void* omega = nullptr;
    double* H = nullptr;                 // warm start of the carbonate solve
    int* fails = nullptr;
    void* drift = nullptr;               // [MAX_NT][Nz+1], compute precision (substep)
    void* wprof = nullptr;               // [2][Nz+1], state precision (the functor's ℑz)
    uint32_t drift_mask = 0;
    NegativesSpec neg;
    const void* u = nullptr;
    const void* v = nullptr;
    bool bound = false;
    int blocks = 0;
    // per-stage CUDA events while profiling: stage start, omega start, functor start, substep start, end
    bool profiling = false;
    bool in_step = false;
    std::vector<cudaEvent_t> ev;
    size_t ev_used = 0;
};

namespace {

int model_free(obgc_pisces_model* m) {
    if (!m) return OBGC_OK;
    for (cudaEvent_t e : m->ev) cudaEventDestroy(e);
    for (int q = 0; q < PNT; q++) { cudaFree(m->scratch[q]); cudaFree(m->G[q]); }
    for (int q = 0; q < OBGC_PIS_NUM_BGC; q++) cudaFree(m->Gb[q]);
    for (int q = 0; q < 4; q++) cudaFree(m->par[q]);
    cudaFree(m->chl); cudaFree(m->zeu); cudaFree(m->mlpar); cudaFree(m->omega); cudaFree(m->H); cudaFree(m->fails);
    cudaFree(m->drift); cudaFree(m->wprof);
    delete m;
    return OBGC_OK;
}

int32_t state_dtype(const obgc_pisces_model* m) { return m->ts == 4 ? OBGC_F32 : OBGC_F64; }

// Records the next profiling event of the step in flight (no-op unless profiling).
int prof_mark(obgc_pisces_model* m, cudaStream_t st) {
    if (!m->profiling || !m->in_step) return OBGC_OK;
    if (m->ev_used == m->ev.size()) {
        cudaEvent_t e;
        OBGC_CUDA(cudaEventCreate(&e));
        m->ev.push_back(e);
    }
    OBGC_CUDA(cudaEventRecord(m->ev[m->ev_used++], st));
    return OBGC_OK;
}

template <typename TS>
int update_state(obgc_pisces_model* m, double t, cudaStream_t st) {
    const obgc_grid& g = m->desc.grid;
    const int64_t N = (int64_t)g.Nx * g.Ny * g.Nz;
    const unsigned blocks = (unsigned)std::min<int64_t>((N + 255) / 256, (int64_t)m->blocks * 8);
    const TS* PChl = static_cast<const TS*>(m->user[OBGC_PIS_PCHL]);
    const TS* DChl = static_cast<const TS*>(m->user[OBGC_PIS_DCHL]);
    chl_sum_kernel<TS><<<blocks, 256, 0, st>>>(PChl, DChl, static_cast<TS*>(m->chl), g.Nx, g.Ny, g.Nz, g.stride_j, g.stride_k);
    OBGC_LAUNCHED("chl_sum_kernel");
    void* bands[4] = {m->par[1], m->par[2], m->par[3], nullptr};
    // light in FP32 arithmetic for the FP32 and mixed paths (FP64 fields for the mixed path), FP64
    // for the plain FP64 path
    int rc = (m->ts == 4 || m->desc.precision == OBGC_PREC_F64) ? obgc_multiband_par(m->desc.nbands, m->desc.kw, m->desc.e, m->desc.chi, m->desc.division,
                                             &m->desc.surface, &g, state_dtype(m), m->chl, bands, m->par[0], t, st)
                        : multiband_par_mixed(m->desc.nbands, m->desc.kw, m->desc.e, m->desc.chi, m->desc.division,
                                              &m->desc.surface, &g, m->chl, bands, m->par[0], t, st);
    if (rc != OBGC_OK) return rc;
    rc = obgc_euphotic_depth(&m->desc.surface, &g, state_dtype(m), m->par[0], m->zeu, 1e-3, t, st);
    if (rc != OBGC_OK) return rc;
    obgc_pisces_field z;
    std::memset(&z, 0, sizeof(z));
    z.kind = OBGC_PF_CONSTANT;
    z.value = m->desc.mixed_layer_depth;
    rc = obgc_mixed_layer_mean(&g, state_dtype(m), m->par[0], &z, m->mlpar, st);
    if (rc != OBGC_OK) return rc;
    rc = prof_mark(m, st);
    if (rc != OBGC_OK) return rc;
    return launch_pisces_omega<TS>(&m->desc.carbon, &g, m->user[OBGC_PIS_DIC], m->user[OBGC_PIS_ALK], m->user[OBGC_PIS_T],
                                   m->user[OBGC_PIS_S], m->user[OBGC_PIS_SI], m->omega, m->H, m->fails, st);
}

int update_state_any(obgc_pisces_model* m, double t, cudaStream_t st) {
    const int rp = prof_mark(m, st);
    if (rp != OBGC_OK) return rp;
    if (m->desc.negatives == OBGC_NEGATIVES_SCALE) {
        const int rc = launch_negatives(m->neg, m->ts, m->user, m->desc.grid, st);
        if (rc != OBGC_OK) return rc;
    }
    return m->ts == 4 ? update_state<float>(m, t, st) : update_state<double>(m, t, st);
}

// The auxiliary inputs of the functor, read from the fields update_state wrote.
void aux_fields(const obgc_pisces_model* m, obgc_pisces_field* a) {
    std::memset(a, 0, sizeof(obgc_pisces_field) * OBGC_PAUX_NUM);
    const int Nz1 = m->desc.grid.Nz + 1;
    a[OBGC_PAUX_ZMXL] = {OBGC_PF_CONSTANT, 0, m->desc.mixed_layer_depth, nullptr};
    a[OBGC_PAUX_ZEU] = {OBGC_PF_XY, 0, 0.0, m->zeu};
    a[OBGC_PAUX_SICLIM] = {OBGC_PF_CONSTANT, 0, m->desc.pisces.silicate_climatology, nullptr};
    a[OBGC_PAUX_OMEGA] = {OBGC_PF_XYZ, 0, 0.0, m->omega};
    a[OBGC_PAUX_KAPPA] = {OBGC_PF_CONSTANT, 0, m->desc.mean_kappa, nullptr};
    a[OBGC_PAUX_MLPAR] = {OBGC_PF_XY, 0, 0.0, m->mlpar};
    a[OBGC_PAUX_WPOC] = {OBGC_PF_ZPROFILE, 0, 0.0, m->wprof};
    a[OBGC_PAUX_WGOC] = {OBGC_PF_ZPROFILE, 0, 0.0, static_cast<char*>(m->wprof) + m->ts * Nz1};
    a[OBGC_PAUX_PAR] = {OBGC_PF_XYZ, 0, 0.0, m->par[0]};
    a[OBGC_PAUX_PAR1] = {OBGC_PF_XYZ, 0, 0.0, m->par[1]};
    a[OBGC_PAUX_PAR2] = {OBGC_PF_XYZ, 0, 0.0, m->par[2]};
    a[OBGC_PAUX_PAR3] = {OBGC_PF_XYZ, 0, 0.0, m->par[3]};
}

// The fused substep launches of one RK3 stage: the 26 tracers advect independently once their BGC
// tendencies are in hand, in launches on tracers 0-8, 9-17 (POC and GOC, slots 1 and 2 of the group,
// keep their register windows) and 18-25, each holding a third of the shared-memory tiles and running
// three blocks per SM.
constexpr int NGROUP = 3;
constexpr int G_FIRST[NGROUP] = {0, 9, 18}, G_SIZE[NGROUP] = {9, 9, 8};

template <typename TS, typename TC>
struct PiscesPlan {
    SubstepArgs<TS, TC> a;
    const FusedEntry* fes[NGROUP];
    int blocks = 0;
    obgc_pisces_field aux[OBGC_PAUX_NUM];
};

template <typename TS, typename TC>
int plan_pisces(obgc_pisces_model* m, double dt, PiscesPlan<TS, TC>& p) {
    for (int q = 0; q < NGROUP; q++) {
        p.fes[q] = find_fused(m->desc.precision, V_EXTERNAL, G_SIZE[q]);
        if (!p.fes[q]) return fail(OBGC_ERR_UNSUPPORTED, "obgc_pisces_model_step: no fused PISCES kernel for this precision");
    }
    const obgc_grid& g = m->desc.grid;
    SubstepArgs<TS, TC>& a = p.a;
    std::memset(&a, 0, sizeof(a));
    a.Nx = g.Nx; a.Ny = g.Ny; a.Nz = g.Nz;
    a.periodic_x = g.topology_x == OBGC_PERIODIC;
    a.periodic_y = g.topology_y == OBGC_PERIODIC;
    a.flat_x = g.topology_x == OBGC_FLAT || !m->desc.advection;
    a.flat_y = g.topology_y == OBGC_FLAT || !m->desc.advection;
    a.sj = g.stride_j; a.sk = g.stride_k;
    a.osj = g.stride_j; a.osk = g.stride_k;
    a.vsj = g.stride_j; a.vsk = g.stride_k;
    a.gsj = g.stride_j; a.gsk = g.stride_k;
    a.dx = TC(g.Lx / g.Nx); a.dy = TC(g.Ly / g.Ny); a.dz = TC(g.Lz / g.Nz); a.Lz = TC(g.Lz);
    a.inv_dx = TC(g.Nx / g.Lx); a.inv_dy = TC(g.Ny / g.Ly); a.inv_dz = TC(g.Nz / g.Lz);
    a.TZ = g.Nz < 8 ? g.Nz : 8;
    a.nseg = (g.Nz + a.TZ - 1) / a.TZ;
    a.ntx = (g.Nx + STEP_BX - 1) / STEP_BX;
    a.nty = (g.Ny + STEP_BY - 1) / STEP_BY;
    a.n_items = a.ntx * a.nty * a.nseg;
    a.u = m->desc.advection ? static_cast<const TS*>(m->u) : nullptr;
    a.v = m->desc.advection ? static_cast<const TS*>(m->v) : nullptr;
    a.w = nullptr;
    a.dt_d = dt;
    a.dt = TC(dt);
    int occ = 1;
    const int rc = p.fes[0]->occupancy(&occ);
    if (rc != OBGC_OK) return rc;
    p.blocks = std::min(a.n_items, m->blocks * (occ > 0 ? occ : 1));
    aux_fields(m, p.aux);
    return OBGC_OK;
}

// One RK3 stage at time ts from the tracers in cur into nxt: update_state! on cur (the negative-tracer
// modifier, light, euphotic depth, mixed-layer PAR, calcite saturation), the functor, then the
// substep launches.  The previous stage's tendencies live in the model (m->G).
template <typename TS, typename TC>
int pisces_stage(obgc_pisces_model* m, PiscesPlan<TS, TC>& p, int stg, double ts, void* const* cur, void* const* nxt,
                 cudaStream_t st) {
    const obgc_grid& g = m->desc.grid;
    SubstepArgs<TS, TC>& a = p.a;
    // update_state! reads the current state: point the model at it for this stage
    void* user_saved[PNT];
    std::memcpy(user_saved, m->user, sizeof(user_saved));
    std::memcpy(m->user, cur, sizeof(user_saved));
    int rc = update_state_any(m, ts, st);
    std::memcpy(m->user, user_saved, sizeof(user_saved));
    if (rc == OBGC_OK) rc = prof_mark(m, st);
    if (rc == OBGC_OK) rc = launch_pisces<TS, TC>(&m->desc.pisces, &g, cur, p.aux, m->Gb, ts, st);
    if (rc == OBGC_OK) rc = prof_mark(m, st);
    if (rc != OBGC_OK) return rc;
    const uint32_t mask = m->desc.advection ? m->drift_mask : 0u;
    a.first_stage = stg == 0;
    a.write_G = stg < 2;
    a.gamma = TC(rk3_gamma(stg));
    a.zeta = TC(rk3_zeta(stg));
    a.c_stage = rk3_c(stg);
    for (int q = 0; q < NGROUP && rc == OBGC_OK; q++) {
        const int g0 = G_FIRST[q], gn = G_SIZE[q];
        for (int t = 0; t < gn; t++) {
            a.in[t] = static_cast<const TS*>(cur[g0 + t]);
            a.out[t] = static_cast<TS*>(nxt[g0 + t]);
            a.G[t] = static_cast<TC*>(m->G[g0 + t]);
            a.ext[t] = g0 + t < OBGC_PIS_NUM_BGC ? static_cast<const TC*>(m->Gb[g0 + t]) : nullptr;
        }
        a.n_ext = std::max(0, std::min(gn, OBGC_PIS_NUM_BGC - g0));
        a.drift = static_cast<const TC*>(m->drift) + (size_t)g0 * (g.Nz + 1);
        a.drift_mask = (mask >> g0) & ((1u << gn) - 1u);
        rc = p.fes[q]->launch(&a, p.blocks, st);
    }
    if (rc == OBGC_OK) rc = prof_mark(m, st);
    return rc;
}

template <typename TS, typename TC>
int enqueue(obgc_pisces_model* m, double t, double dt, int nsteps, cudaStream_t st) {
    PiscesPlan<TS, TC> p;
    int rc = plan_pisces<TS, TC>(m, dt, p);
    if (rc != OBGC_OK) return rc;
    const obgc_grid& g = m->desc.grid;
    void* cur[PNT];
    void* nxt[PNT];
    for (int q = 0; q < PNT; q++) { cur[q] = m->user[q]; nxt[q] = m->scratch[q]; }
    for (int s = 0; s < nsteps && rc == OBGC_OK; s++) {
        for (int stg = 0; stg < 3 && rc == OBGC_OK; stg++) {
            rc = pisces_stage<TS, TC>(m, p, stg, t + s * dt + rk3_c(stg) * dt, cur, nxt, st);
            for (int q = 0; q < PNT; q++) { void* tmp = cur[q]; cur[q] = nxt[q]; nxt[q] = tmp; }
        }
    }
    if (rc != OBGC_OK) return rc;
    if (m->desc.negatives == OBGC_NEGATIVES_SCALE) {
        rc = launch_negatives(m->neg, m->ts, cur, g, st);   // update_state! after the last substep
        if (rc != OBGC_OK) return rc;
    }
    if (nsteps % 2 == 1) {
        CopyFields<TS> F;
        for (int q = 0; q < PNT; q++) { F.src[q] = static_cast<const TS*>(cur[q]); F.dst[q] = static_cast<TS*>(m->user[q]); }
        const int64_t N = (int64_t)g.Nx * g.Ny * g.Nz;
        copy_fields_kernel<TS><<<(unsigned)std::min<int64_t>((N + 255) / 256, (int64_t)m->blocks * 8), 256, 0, st>>>(
            F, g.Nx, g.Ny, g.Nz, g.stride_j, g.stride_k);
        OBGC_LAUNCHED("copy_fields_kernel");
    }
    return OBGC_OK;
}

// One stage from caller arrays `in` into `out` (the model's grid layout), and with `finish` the
// modifier that ends a call.
template <typename TS, typename TC>
int enqueue_one(obgc_pisces_model* m, double t, double dt, int stage, void* const* in, void* const* out, bool finish,
                cudaStream_t st) {
    PiscesPlan<TS, TC> p;
    int rc = plan_pisces<TS, TC>(m, dt, p);
    if (rc == OBGC_OK) rc = pisces_stage<TS, TC>(m, p, stage, t + rk3_c(stage) * dt, in, out, st);
    if (rc == OBGC_OK && finish && m->desc.negatives == OBGC_NEGATIVES_SCALE)
        rc = launch_negatives(m->neg, m->ts, const_cast<void**>(out), m->desc.grid, st);
    return rc;
}

template <typename TS, typename TC>
int build_profiles(obgc_pisces_model* m) {
    const obgc_grid& g = m->desc.grid;
    const obgc_pisces_params& p = m->desc.pisces;
    const int Nz = g.Nz, Nz1 = Nz + 1;
    const double dz = g.Lz / Nz;
    std::vector<double> wpoc(Nz1), wgoc(Nz1);
    for (int f = 0; f < Nz1; f++) {
        wpoc[f] = f < Nz ? -p.poc_sinking_speed * (p.open_bottom ? 1.0 : 1.0 - std::exp(-f / 2.0)) : 0.0;
        const double zc = -g.Lz + (f + 0.5) * dz;
        const double zm = std::min(m->desc.mixed_layer_depth, 0.0);
        wgoc[f] = f < Nz ? -p.goc_minimum_speed + (p.goc_maximum_speed - p.goc_minimum_speed) * std::min(0.0, zc - zm) / 5000 : 0.0;
    }
    std::vector<TC> drift((size_t)MAX_NT * Nz1, TC(0));
    const int poc_slots[2] = {OBGC_PIS_POC, OBGC_PIS_SFE};
    const int goc_slots[4] = {OBGC_PIS_GOC, OBGC_PIS_BFE, OBGC_PIS_PSI, OBGC_PIS_CACO3};
    m->drift_mask = 0;
    for (int q : poc_slots) {
        for (int f = 0; f < Nz1; f++) drift[(size_t)q * Nz1 + f] = TC(wpoc[f]);
        if (p.poc_sinking_speed != 0.0) m->drift_mask |= 1u << q;
    }
    for (int q : goc_slots) {
        for (int f = 0; f < Nz1; f++) drift[(size_t)q * Nz1 + f] = TC(wgoc[f]);
        m->drift_mask |= 1u << q;
    }
    std::vector<TS> prof((size_t)2 * Nz1);
    for (int f = 0; f < Nz1; f++) { prof[f] = TS(wpoc[f]); prof[Nz1 + f] = TS(wgoc[f]); }
    OBGC_CUDA(cudaMemcpy(m->drift, drift.data(), sizeof(TC) * drift.size(), cudaMemcpyHostToDevice));
    OBGC_CUDA(cudaMemcpy(m->wprof, prof.data(), sizeof(TS) * prof.size(), cudaMemcpyHostToDevice));
    return OBGC_OK;
}

}  // namespace

extern "C" int obgc_pisces_model_create(const obgc_pisces_model_desc* d, obgc_pisces_model** out) {
    if (!d || !out) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_create: null argument");
    *out = nullptr;
    if (!valid_grid(&d->grid) || (d->precision < OBGC_PREC_F32 || d->precision > OBGC_PREC_MIXED) || d->nbands != 3 || (d->negatives != OBGC_NEGATIVES_NONE && d->negatives != OBGC_NEGATIVES_SCALE) ||
        (d->surface.kind != OBGC_SURFACE_PAR_DEFAULT && d->surface.kind != OBGC_SURFACE_PAR_CONSTANT) || !(d->mean_kappa > 0))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_create: bad descriptor");
    double sum = 0;
    for (int b = 0; b < d->nbands; b++) sum += d->division[b];
    if (sum != 1.0) return fail(OBGC_ERR_INVALID_ARGUMENT, "surface_PAR_division does not sum to 1");
    obgc_pisces_model* m = new obgc_pisces_model();
    m->desc = *d;
    m->ts = d->precision == OBGC_PREC_F32 ? 4 : 8;
    m->tc = d->precision == OBGC_PREC_F64 ? 8 : 4;
    const obgc_grid& g = d->grid;
    m->extent = g.stride_k * (int64_t)g.Nz;
    const int64_t xy = (int64_t)g.Nx * g.Ny;
    int rc = OBGC_OK;
    auto alloc = [&](void** p, size_t bytes) {
        if (rc != OBGC_OK) return;
        const cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc(PISCES model)");
    };
    for (int q = 0; q < PNT; q++) {
        alloc(&m->scratch[q], m->ts * m->extent);
        alloc(&m->G[q], m->tc * m->extent);
    }
    for (int q = 0; q < OBGC_PIS_NUM_BGC; q++) alloc(&m->Gb[q], m->tc * m->extent);
    for (int q = 0; q < 4; q++) alloc(&m->par[q], m->ts * m->extent);
    alloc(&m->chl, m->ts * m->extent);
    alloc(&m->zeu, m->ts * xy);
    alloc(&m->mlpar, m->ts * xy);
    alloc(&m->omega, m->ts * m->extent);
    alloc((void**)&m->H, sizeof(double) * (size_t)xy * g.Nz);
    alloc((void**)&m->fails, sizeof(int));
    alloc(&m->drift, m->tc * (size_t)MAX_NT * (g.Nz + 1));
    alloc(&m->wprof, m->ts * 2 * (size_t)(g.Nz + 1));
    if (rc == OBGC_OK && cudaMemset(m->H, 0, sizeof(double) * (size_t)xy * g.Nz) != cudaSuccess)
        rc = fail(OBGC_ERR_CUDA, "cudaMemset(H)");
    if (rc == OBGC_OK)
        rc = m->ts == 4 ? build_profiles<float, float>(m)
                        : m->tc == 8 ? build_profiles<double, double>(m) : build_profiles<double, float>(m);
    m->neg = pisces_negatives_spec(d->pisces, d->invalid_fill_value);
    int dev = 0, nsm = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    m->blocks = nsm;
    if (rc != OBGC_OK) { model_free(m); return rc; }
    *out = m;
    return OBGC_OK;
}

extern "C" int obgc_pisces_model_destroy(obgc_pisces_model* m) { return model_free(m); }

extern "C" int obgc_pisces_model_bind(obgc_pisces_model* m, void* const* tracers, const void* u, const void* v) {
    if (!m || !tracers) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_bind: null argument");
    for (int q = 0; q < PNT; q++) {
        if (!tracers[q]) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_bind: a tracer field is NULL");
        m->user[q] = tracers[q];
    }
    m->u = u;
    m->v = v;
    m->bound = true;
    return OBGC_OK;
}

extern "C" int obgc_pisces_model_update_state(obgc_pisces_model* m, double t, void* stream) {
    if (!m || !m->bound) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_update_state: model not bound");
    return update_state_any(m, t, static_cast<cudaStream_t>(stream));
}

extern "C" int obgc_pisces_model_step(obgc_pisces_model* m, double t, double dt, int32_t nsteps, void* stream) {
    if (!m || !m->bound || nsteps < 0 || !(dt > 0)) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_step: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    m->ev_used = 0;
    m->in_step = true;
    const int rc = m->ts == 4 ? enqueue<float, float>(m, t, dt, nsteps, st)
                   : m->tc == 8 ? enqueue<double, double>(m, t, dt, nsteps, st) : enqueue<double, float>(m, t, dt, nsteps, st);
    m->in_step = false;
    if (rc != OBGC_OK) m->ev_used = 0;
    return rc;
}

extern "C" int obgc_pisces_model_substep(obgc_pisces_model* m, double t, double dt, int32_t stage, const void* const* in,
                                         void* const* out, int32_t finish, void* stream) {
    if (!m || !m->bound || stage < 0 || stage > 2 || !(dt > 0) || !in || !out)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_substep: bad argument");
    for (int q = 0; q < PNT; q++)
        if (!in[q] || !out[q] || in[q] == out[q])
            return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_substep: every tracer needs distinct input and output arrays");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    void* const* vin = const_cast<void* const*>(in);
    m->ev_used = 0;
    m->in_step = true;
    const int rc = m->ts == 4 ? enqueue_one<float, float>(m, t, dt, stage, vin, out, finish != 0, st)
                   : m->tc == 8 ? enqueue_one<double, double>(m, t, dt, stage, vin, out, finish != 0, st)
                                : enqueue_one<double, float>(m, t, dt, stage, vin, out, finish != 0, st);
    m->in_step = false;
    if (rc != OBGC_OK) m->ev_used = 0;
    return rc;
}

extern "C" int obgc_pisces_model_set_profiling(obgc_pisces_model* m, int32_t on) {
    if (!m) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_set_profiling: null model");
    m->profiling = on != 0;
    m->ev_used = 0;
    return OBGC_OK;
}

extern "C" int obgc_pisces_model_last_timing(obgc_pisces_model* m, double* ms, int32_t* stages) {
    if (!m || !ms) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_last_timing: null argument");
    for (int q = 0; q < 4; q++) ms[q] = 0.0;
    const size_t n = m->ev_used / 5;
    if (stages) *stages = (int32_t)n;
    if (n == 0) return OBGC_OK;
    OBGC_CUDA(cudaEventSynchronize(m->ev[5 * n - 1]));
    for (size_t s = 0; s < n; s++)
        for (int q = 0; q < 4; q++) {
            float x = 0.f;
            OBGC_CUDA(cudaEventElapsedTime(&x, m->ev[5 * s + q], m->ev[5 * s + q + 1]));
            ms[q] += x;
        }
    return OBGC_OK;
}

extern "C" int obgc_pisces_model_field(obgc_pisces_model* m, int32_t which, void** ptr) {
    if (!m || !ptr) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_field: null argument");
    switch (which) {
        case OBGC_PMF_PAR: case OBGC_PMF_PAR1: case OBGC_PMF_PAR2: case OBGC_PMF_PAR3: *ptr = m->par[which]; return OBGC_OK;
        case OBGC_PMF_ZEU: *ptr = m->zeu; return OBGC_OK;
        case OBGC_PMF_MLPAR: *ptr = m->mlpar; return OBGC_OK;
        case OBGC_PMF_OMEGA: *ptr = m->omega; return OBGC_OK;
    }
    return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_field: unknown field");
}

extern "C" int obgc_pisces_model_read_field(obgc_pisces_model* m, int32_t which, double* out) {
    void* p = nullptr;
    const int rc = obgc_pisces_model_field(m, which, &p);
    if (rc != OBGC_OK) return rc;
    if (!out) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_model_read_field: null output");
    const obgc_grid& g = m->desc.grid;
    const bool xy = which == OBGC_PMF_ZEU || which == OBGC_PMF_MLPAR;
    const size_t n = xy ? (size_t)g.Nx * g.Ny : (size_t)m->extent;
    std::vector<char> host(n * m->ts);
    OBGC_CUDA(cudaDeviceSynchronize());
    OBGC_CUDA(cudaMemcpy(host.data(), p, host.size(), cudaMemcpyDeviceToHost));
    auto at = [&](size_t q) { return m->ts == 4 ? (double)reinterpret_cast<const float*>(host.data())[q]
                                                : reinterpret_cast<const double*>(host.data())[q]; };
    if (xy) {
        for (size_t q = 0; q < n; q++) out[q] = at(q);
        return OBGC_OK;
    }
    size_t o = 0;
    for (int k = 0; k < g.Nz; k++)
        for (int j = 0; j < g.Ny; j++)
            for (int i = 0; i < g.Nx; i++) out[o++] = at((size_t)i + (size_t)j * g.stride_j + (size_t)k * g.stride_k);
    return OBGC_OK;
}

