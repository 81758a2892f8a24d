// step.cu — the 3-D model context: fused RK3 stepping (mode (ii)), the plugin hooks of mode (i)
// (update_state / compute_tendencies), CUDA-graph replay, and the FP64 compensated tracer budget.
#include <cudaTypedefs.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>
#include "gas_device.cuh"
#include "multig_device.cuh"
#include "negatives.cuh"
#include "step_launch.cuh"

namespace obgc {

template <typename T>
int launch_gas_exchange_multi(const GasMulti& m, const obgc_grid* grid, const void* Tc, const void* S, cudaStream_t st);
bool valid_gas(const obgc_gas_exchange* g);

// ----------------------------------------------------------------------------- registry
static std::vector<FusedEntry>& registry() {
    static std::vector<FusedEntry> r;
    return r;
}
static std::mutex& registry_mutex() {
    static std::mutex m;
    return m;
}
void register_fused(const FusedEntry& e) {
    std::lock_guard<std::mutex> g(registry_mutex());
    registry().push_back(e);
}
const FusedEntry* find_fused(int prec, int V, int NT) {
    std::lock_guard<std::mutex> g(registry_mutex());
    for (const auto& e : registry())
        if (e.prec == prec && e.V == V && e.NT == NT) return &e;
    return nullptr;
}

int required_tracers(const obgc_npd_params* p, int32_t* names);
bool drift_speed(const obgc_npd_params* p, int name, double* w0);
void drift_profile(double w0, int open_bottom, int Nz, double* w);

// ----------------------------------------------------------------------------- small kernels
__global__ void set_time_kernel(double* t, double v, int* status) {
    *t = v;
    if (status) *status = 0;
}
__global__ void advance_time_kernel(double* t, double dt) { *t += dt; }

// SimpleMultiGSediment, one thread per column after every RK3 stage of the water (and once before a
// call's first stage with dt = 0): track the bottom cells of the new state, step the sediment fields
// a full RK3 step of dt (the first stage from the tendency cached at the end of the previous step;
// afresh on the first step), cache the final tendency, and write the coupled bottom-cell tendencies
// for the next water stage.
template <typename TS>
struct MultiGArgs {
    MultiG m;
    int Nx, Ny;
    int64_t sj;                 // the bottom level (k = 0) of the state arrays: i + j sj
    int n_sink;
    const TS* sink[4];          // sinking tracers
    double w0[4];               // their drift velocity at the bottom face (negative: downward)
    const TS* no3;
    const TS* nh4;
    const TS* o2;
    double* state;              // [4][Ny Nx]: Ns, Nf, Nr, started (0 / 1)
    double* gcache;             // [3][Ny Nx]: the fields' tendency at the end of the last step
    double* flux;               // [3][Ny Nx]: coupled tendencies of NO3, NH4, O2 (mmol/m2/s)
    double dt;                  // step length (0: the coupled tendencies only)
};

template <typename TS>
__global__ void __launch_bounds__(128) multig_kernel(const __grid_constant__ MultiGArgs<TS> a) {
    const int64_t NN = (int64_t)a.Nx * a.Ny;
    const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= NN) return;
    const int i = (int)(col % a.Nx), j = (int)(col / a.Nx);
    const int64_t o = i + (int64_t)j * a.sj;
    // sinking_flux (tracked_fields.jl:55-70): minus the advective flux through the bottom face,
    // whose face value next to the wall is the bottom cell's
    double dep = 0.0;
    for (int q = 0; q < a.n_sink; q++) dep -= a.w0[q] * (double)a.sink[q][o];
    double* S = a.state;
    double s0 = S[col], s1 = S[NN + col], s2 = S[2 * NN + col];
    if (a.dt > 0.0) {
        const double g[3] = {8.0 / 15.0, 5.0 / 12.0, 3.0 / 4.0}, z[3] = {0.0, -17.0 / 60.0, -5.0 / 12.0};
        double G0[3], G1[3];
        if (S[3 * NN + col] == 0.0) {
            multig_fields_tendency(a.m, s0, s1, dep, G0);
            S[3 * NN + col] = 1.0;
        } else {
            for (int q = 0; q < 3; q++) G0[q] = a.gcache[q * NN + col];
        }
        double x[3] = {s0, s1, s2};
        for (int q = 0; q < 3; q++) x[q] += a.dt * g[0] * G0[q];
        multig_fields_tendency(a.m, x[0], x[1], dep, G1);
        for (int q = 0; q < 3; q++) x[q] += a.dt * (g[1] * G1[q] + z[1] * G0[q]);
        multig_fields_tendency(a.m, x[0], x[1], dep, G0);
        for (int q = 0; q < 3; q++) x[q] += a.dt * (g[2] * G0[q] + z[2] * G1[q]);
        multig_fields_tendency(a.m, x[0], x[1], dep, G1);
        for (int q = 0; q < 3; q++) a.gcache[q * NN + col] = G1[q];
        s0 = x[0]; s1 = x[1]; s2 = x[2];
        S[col] = s0; S[NN + col] = s1; S[2 * NN + col] = s2;
    }
    double F0, F1, F2;
    multig_coupling(a.m, s0, s1, (double)a.no3[o], (double)a.nh4[o], (double)a.o2[o], &F0, &F1, &F2);
    a.flux[col] = F0;
    a.flux[NN + col] = F1;
    a.flux[2 * NN + col] = F2;
}

// Thomas factors of the vertically implicit diffusion for the three RK3 stages (the same in every
// column): out[(2 st) Nz + k] = c'_k and out[(2 st + 1) Nz + k] = 1 / pivot_k of
// (I - dt_s d/dz kappa d/dz), dt_s = (gamma_st + zeta_st) dt; lo_k = -r kappa_k (face below k,
// zero at the bottom wall), up_k = -r kappa_(k+1) (zero at the top wall), r = dt_s / dz^2.
__global__ void thomas_factors_kernel(const double* __restrict__ kappa_faces, int Nz, double inv_dz2, double dt,
                                      double* __restrict__ out) {
    const int st = threadIdx.x;
    if (st >= 3) return;
    const double r = (rk3_gamma(st) + rk3_zeta(st)) * dt * inv_dz2;
    double cprev = 0.0;
    for (int k = 0; k < Nz; k++) {
        const double lo = k > 0 ? -r * kappa_faces[k] : 0.0;
        const double up = k < Nz - 1 ? -r * kappa_faces[k + 1] : 0.0;
        const double den = (1.0 - lo - up) - lo * cprev;
        cprev = up / den;
        out[(2 * st) * Nz + k] = cprev;
        out[(2 * st + 1) * Nz + k] = 1.0 / den;
    }
}

template <typename TS>
struct ImplicitFields {
    TS* f[MAX_NT];
};

// One thread per (column, tracer): forward sweep d_k = (x_k - lo_k d_(k-1)) / pivot_k in place,
// then x_k = d_k - c'_k x_(k+1).  Threads of a warp take neighbouring columns, so every level's
// loads and stores are coalesced.
template <typename TS>
__global__ void implicit_vertical_kernel(const __grid_constant__ ImplicitFields<TS> F, int nslots, int Nx, int Ny, int Nz,
                                         int64_t sj, int64_t sk, const double* __restrict__ kappa_faces, double inv_dz2,
                                         double dt, int st, const double* __restrict__ factors) {
    const int64_t NN = (int64_t)Nx * Ny;
    const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= NN * nslots) return;
    const int t = (int)(g / NN);
    const int64_t c = g - (int64_t)t * NN;
    TS* x = F.f[t] + (c % Nx) + (c / Nx) * sj;
    const double r = (rk3_gamma(st) + rk3_zeta(st)) * dt * inv_dz2;
    const double* cp = factors + (2 * st) * Nz;
    const double* ip = factors + (2 * st + 1) * Nz;
    double d = 0.0;
    for (int k = 0; k < Nz; k++) {
        const double lo = k > 0 ? -r * kappa_faces[k] : 0.0;
        d = ((double)x[k * sk] - lo * d) * ip[k];
        x[k * sk] = TS(d);
    }
    double xn = d;
    for (int k = Nz - 2; k >= 0; k--) {
        xn = (double)x[k * sk] - cp[k] * xn;
        x[k * sk] = TS(xn);
    }
}

template <typename TS>
__global__ void copy_interior_kernel(const TS* __restrict__ src, TS* __restrict__ dst, int Nx, int Ny, int Nz,
                                     int64_t sj, int64_t sk) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t NN = (int64_t)Nx * Ny;
    if (c >= NN * Nz) return;
    const int64_t idx = (c % Nx) + ((c / Nx) % Ny) * sj + (c / NN) * sk;
    dst[idx] = src[idx];
}

// The caller's arrays copied into a padded set (x halo TMA_HX, y halo HALO, rows of pad_sj values)
// with the periodic images in the halos, so that the first TMA-staged stage of a call copies every
// tile with tensor copies.  One thread per padded cell and level, every slot; halo cells of a
// Bounded direction and the row tails past Nx + 2 TMA_HX are left as they are (no stencil reads
// them).
template <typename TS>
struct PadCopyArgs {
    const TS* src[MAX_NT];
    float* dst[MAX_NT];           // the padded arrays' first cell (x = -TMA_HX, y = -HALO)
    int nt;
};
// Whether padded cell (px, py) lies in the box of a tile that needs the periodic wrap (tile (ti, tj)
// copies padded x in [32 ti, 32 ti + 40) and y in [8 tj, 8 tj + 14)).
__device__ inline bool in_wrapping_box(int px, int py, int Nx, int Ny, bool periodic_x, bool periodic_y) {
    const int ntx = (Nx + STEP_BX - 1) / STEP_BX, nty = (Ny + STEP_BY - 1) / STEP_BY;
    const int ti1 = min(px / STEP_BX, ntx - 1), tj1 = min(py / STEP_BY, nty - 1);
    const int ti0 = px >= TMA_TILE_W ? (px - TMA_TILE_W) / STEP_BX + 1 : 0;
    const int tj0 = py >= TILE_H ? (py - TILE_H) / STEP_BY + 1 : 0;
    for (int tj = tj0; tj <= tj1; tj++)
        for (int ti = ti0; ti <= ti1; ti++)
            if (tile_wraps_xy(ti * STEP_BX, tj * STEP_BY, Nx, Ny, periodic_x, periodic_y)) return true;
    return false;
}
// FP64 state (the mixed path) is rounded to FP32 on the way, as the cp.async staging rounds it.
// bands: only the cells of the boxes of the tiles that need the wrap (the call's first stage copies
// the other tiles from the caller's arrays).
template <typename TS>
__global__ void pad_copy_kernel(PadCopyArgs<TS> p, int Nx, int Ny, int Nz, int64_t sj, int64_t sk, int64_t psj, int64_t psk,
                                int periodic_x, int periodic_y, int bands) {
    const int PW = Nx + 2 * TMA_HX, PH = Ny + 2 * HALO;
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (int64_t)PW * PH * Nz) return;
    const int px = (int)(c % PW), py = (int)((c / PW) % PH), k = (int)(c / ((int64_t)PW * PH));
    if (bands && !in_wrapping_box(px, py, Nx, Ny, periodic_x, periodic_y)) return;
    int x = px - TMA_HX, y = py - HALO;
    if (x < 0 || x >= Nx) {
        if (!periodic_x) return;
        x = x < 0 ? x + Nx : x - Nx;
    }
    if (y < 0 || y >= Ny) {
        if (!periodic_y) return;
        y = y < 0 ? y + Ny : y - Ny;
    }
    const int64_t s = x + (int64_t)y * sj + (int64_t)k * sk, d = px + (int64_t)py * psj + (int64_t)k * psk;
    for (int t = 0; t < p.nt; t++) p.dst[t][d] = float(__ldg(p.src[t] + s));
}

// Neumaier-compensated FP64 accumulation (sum, compensation).
struct DD {
    double s, c;
};
__device__ __forceinline__ void dd_add(DD& a, double x) {
    const double t = a.s + x;
    if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
    else a.c += (x - t) + a.s;
    a.s = t;
}
__device__ __forceinline__ void dd_merge(DD& a, const DD& b) {
    dd_add(a, b.s);
    a.c += b.c;
}

constexpr int BUDGET_MAX_TRACERS = 8;
template <typename TS>
struct BudgetArgs {
    const TS* f[BUDGET_MAX_TRACERS];
    double scale[BUDGET_MAX_TRACERS];
    int n;
};

constexpr int BUDGET_THREADS = 256;
template <typename TS>
__global__ void __launch_bounds__(BUDGET_THREADS) budget_partial_kernel(BudgetArgs<TS> b, int Nx, int Ny, int Nz,
                                                                        int64_t sj, int64_t sk, DD* __restrict__ partial) {
    const int64_t NN = (int64_t)Nx * Ny, N = NN * Nz;
    DD acc = {0.0, 0.0};
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t idx = (c % Nx) + ((c / Nx) % Ny) * sj + (c / NN) * sk;
        for (int q = 0; q < b.n; q++) dd_add(acc, b.scale[q] * (double)b.f[q][idx]);
    }
    __shared__ DD red[BUDGET_THREADS];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = BUDGET_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) dd_merge(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(BUDGET_THREADS) budget_final_kernel(const DD* __restrict__ partial, int n, double* out) {
    DD acc = {0.0, 0.0};
    for (int q = threadIdx.x; q < n; q += blockDim.x) dd_merge(acc, partial[q]);
    __shared__ DD red[BUDGET_THREADS];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = BUDGET_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) dd_merge(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0].s + red[0].c;
}

}  // namespace obgc

using namespace obgc;

// ----------------------------------------------------------------------------- context
struct obgc_ctx {
    obgc_model_desc desc;
    int V = -1, NT = 0, NB = 0;
    int names[MAX_NT];
    int prec = 0;
    size_t ts = 4, tc = 4;
    int64_t extent = 0;                 // elements spanned by one field (strides * Nz)
    obgc_fields fields;
    void* user[MAX_NT] = {};
    void* scratch[MAX_NT] = {};
    void* G[MAX_NT] = {};
    void* drift = nullptr;
    uint32_t drift_mask = 0;
    NegativesSpec neg;                  // negative-tracer modifier over the main slots
    // passive tracers: slots NT .. NT + NP - 1 (names OBGC_PASSIVE(p)), stepped by the
    // external-tendency kernel in launches of 4, 2 and 1 (pchunk); psrc[p]: the named tracer whose
    // BGC tendency passive p takes (OBGC_DIC / OBGC_ALK for CarbonateSystem replicates), or -1
    int NP = 0;
    int psrc[OBGC_MAX_PASSIVE];
    int nchunk = 0;
    int pchunk[OBGC_MAX_PASSIVE];
    int pblocks[5] = {0, 0, 0, 0, 0};   // persistent grid of the 1-, 2- and 4-tracer launches
    NegativesSpec neg_passive;          // ZeroNegativeTracers over the passive slots (else off)
    void* bgc_out[2] = {nullptr, nullptr};   // BGC tendencies of DIC and Alk (compute precision)
    // air-sea gas exchange (top boundary conditions), one per target slot
    struct GasCond {
        bool on = false;
        obgc_gas_exchange g;
        int target = -1, dic = -1, alk = -1;   // slots
        double* flux = nullptr;                 // (Nx, Ny) per stage
        double* H = nullptr;                    // (Nx, Ny): each column's [H+] from the previous stage
    } gas[OBGC_MAX_GAS_CONDITIONS];
    // forcings (prescribed source-rate fields), one per target slot
    struct ForcingSpec {
        int slot = -1;
        const void* rate = nullptr;
        double t0 = 0, t1 = 0;
    } frc[OBGC_MAX_FORCINGS];
    // ScalarDiffusivity (explicit): horizontal kappa, and kappa / dz^2 at the Nz + 1 faces (device,
    // compute precision), or nullptr
    double kappa_h = 0.0;
    void* kzz = nullptr;
    // VerticallyImplicitTimeDiscretization: kappa at the faces (FP64, device, nullptr: no vertical
    // diffusivity) and the Thomas factors of the three stages
    bool vimplicit = false;
    double* kzf = nullptr;
    double* thomas = nullptr;
    // InstantRemineralisation sediment: receiver slot (-1: none), sinking slots, parameters, and the
    // storage (state precision) and previous-stage burial (compute precision) of every column
    int sed_recv = -1;
    uint32_t sed_mask = 0;
    double sed_a = 0, sed_b = 0, sed_k = 0;
    void* sed_storage = nullptr;
    void* sed_G = nullptr;
    // SimpleMultiGSediment (none when mg_on is false)
    bool mg_on = false;
    MultiG mg;
    int mg_nsink = 0;
    int mg_sink[4] = {-1, -1, -1, -1};
    double mg_w0[4] = {0, 0, 0, 0};
    int mg_no3 = -1, mg_nh4 = -1, mg_o2 = -1;
    double* mg_state = nullptr;        // [4][Ny Nx]
    double* mg_gcache = nullptr;       // [3][Ny Nx]
    double* mg_flux = nullptr;         // [3][Ny Nx]
    double* d_time = nullptr;
    int* d_status = nullptr;            // OBGC_FLAG_* of the current call (device)
    int* h_status = nullptr;            // its copy behind the call's last kernel (pinned host)
    bool status_check = true;           // obgc_step waits and returns the status
    DD* partial = nullptr;
    int n_partial = 0;
    double* d_budget = nullptr;
    // tensor-memory-accelerator staging (FP32 state, no passive tracers): two padded copies of every
    // slot (x halo TMA_HX, y halo HALO cells, rows of pad_sj values), the tensor maps of both sets
    // (device), the staging choice (1: TMA when a launch qualifies, 0: cp.async) and what the last
    // obgc_step used
    void* pad[2][MAX_NT] = {};
    CUtensorMap* d_tmaps = nullptr;     // [2][MAX_NT]: the padded sets; [2 MAX_NT + t]: the bound arrays
    void* tma_encode = nullptr;         // the driver's cuTensorMapEncodeTiled
    bool umaps_ok = false;              // the bound arrays have tensor maps (16-byte aligned layout)
    int64_t pad_sj = 0, pad_sk = 0;
    bool tma_ready = false;
    int staging = 1;
    bool last_used_tma = false;
    int TZ = 0;                         // levels per work item; 0: chosen per grid (fill_args)
    bool copied_first = false;          // the last TMA-staged dispatch copied the caller's arrays into a padded set
    // the chlorophyll sums above each segment (par_prefix_kernel), room for par_prefix_segs segments
    // below the first (enough for any segment length of two levels or more), and whether the last
    // dispatch launched the pre-pass
    void* par_prefix = nullptr;
    int par_prefix_segs = 0;
    bool prefix_on = false;
    // the window slots' vertical face fluxes of the TMA-staged stages (sink_flux_kernel), and
    // whether the last dispatch launched that pre-pass
    void* fz_pre = nullptr;
    bool sinkpre_on = false;
    int blocks = 0;
    bool bound = false;
    // graph replay
    cudaGraphExec_t graph = nullptr;
    double graph_dt = 0;
    int graph_nsteps = 0;
    uint64_t bind_version = 0, graph_version = ~0ull;
    cudaStream_t graph_stream = nullptr;
    // timing
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;
    // the TMA-staged stages' side stream: the chlorophyll-sum pre-pass runs there beside the
    // sinking-flux pre-pass (both read the stage's input, each writes its own buffer)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::vector<cudaEvent_t> prof_events;
    bool profile = false;
    double last_total_ms = 0, last_substep_ms = 0;
    int64_t last_launches = 0;
};

static int ctx_free(obgc_ctx* c) {
    if (!c) return OBGC_OK;
    if (c->graph) cudaGraphExecDestroy(c->graph);
    for (int t = 0; t < MAX_NT; t++) {   // main and passive slots
        if (c->scratch[t]) cudaFree(c->scratch[t]);
        if (c->G[t]) cudaFree(c->G[t]);
    }
    if (c->drift) cudaFree(c->drift);
    if (c->par_prefix) cudaFree(c->par_prefix);
    if (c->fz_pre) cudaFree(c->fz_pre);
    if (c->d_time) cudaFree(c->d_time);
    if (c->d_status) cudaFree(c->d_status);
    for (int q = 0; q < 2; q++)
        for (int t = 0; t < MAX_NT; t++)
            if (c->pad[q][t]) cudaFree(c->pad[q][t]);
    if (c->d_tmaps) cudaFree(c->d_tmaps);
    if (c->h_status) cudaFreeHost(c->h_status);
    if (c->partial) cudaFree(c->partial);
    if (c->d_budget) cudaFree(c->d_budget);
    for (auto& gc : c->gas) {
        if (gc.flux) cudaFree(gc.flux);
        if (gc.H) cudaFree(gc.H);
    }
    for (int q = 0; q < 2; q++)
        if (c->bgc_out[q]) cudaFree(c->bgc_out[q]);
    if (c->kzz) cudaFree(c->kzz);
    if (c->kzf) cudaFree(c->kzf);
    if (c->thomas) cudaFree(c->thomas);
    if (c->sed_storage) cudaFree(c->sed_storage);
    if (c->sed_G) cudaFree(c->sed_G);
    if (c->mg_state) cudaFree(c->mg_state);
    if (c->mg_gcache) cudaFree(c->mg_gcache);
    if (c->mg_flux) cudaFree(c->mg_flux);
    if (c->ev_begin) cudaEventDestroy(c->ev_begin);
    if (c->ev_end) cudaEventDestroy(c->ev_end);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->side) cudaStreamDestroy(c->side);
    for (auto e : c->prof_events) cudaEventDestroy(e);
    delete c;
    return OBGC_OK;
}

// The padded slot copies and their tensor maps (3-D: the padded row, the padded rows, the levels;
// box TMA_TILE_W x TILE_H x 1 in FP32).  Without the driver's encoder the context keeps cp.async
// staging (obgc_get_staging reports it).
static int setup_tma(obgc_ctx* c) {
    const obgc_grid& g = c->desc.grid;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return OBGC_OK;
    }
    auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    const size_t bytes = sizeof(float) * (size_t)c->pad_sk * g.Nz;
    c->tma_encode = fn;
    std::vector<CUtensorMap> maps(3 * MAX_NT);
    std::memset(maps.data(), 0, sizeof(CUtensorMap) * maps.size());
    for (int s = 0; s < 2; s++)
        for (int t = 0; t < c->NT; t++) {
            cudaError_t e = cudaMalloc(&c->pad[s][t], bytes);
            if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(padded slot)");
            e = cudaMemset(c->pad[s][t], 0, bytes);
            if (e != cudaSuccess) return cuda_fail(e, "cudaMemset(padded slot)");
            const cuuint64_t dims[3] = {(cuuint64_t)c->pad_sj, (cuuint64_t)(g.Ny + 2 * HALO), (cuuint64_t)g.Nz};
            const cuuint64_t strides[2] = {(cuuint64_t)c->pad_sj * sizeof(float), (cuuint64_t)c->pad_sk * sizeof(float)};
            const cuuint32_t box[3] = {(cuuint32_t)TMA_TILE_W, (cuuint32_t)TILE_H, 1};
            const cuuint32_t es[3] = {1, 1, 1};
            const CUresult r = encode(&maps[(size_t)s * MAX_NT + t], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, c->pad[s][t], dims,
                                      strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                      CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
            if (r != CUDA_SUCCESS) return fail(OBGC_ERR_CUDA, "cuTensorMapEncodeTiled(padded slot) failed: " + std::to_string((int)r));
        }
    cudaError_t e = cudaMalloc(&c->d_tmaps, sizeof(CUtensorMap) * maps.size());
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(tensor maps)");
    // the sinking tracers' face fluxes of the TMA-staged stages
    if (c->drift_mask & ((1u << window_a(c->V)) | (1u << window_b(c->V)))) {
        e = cudaMalloc(&c->fz_pre, sizeof(float) * 2 * (size_t)(g.Nz + 1) * g.Nx * g.Ny);
        if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(sinking fluxes)");
    }
    e = cudaMemcpy(c->d_tmaps, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(tensor maps)");
    c->tma_ready = true;
    return OBGC_OK;
}

extern "C" int obgc_create(const obgc_model_desc* desc, obgc_ctx** out) {
    if (!desc || !out) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_create: null argument");
    *out = nullptr;
    const obgc_grid& g = desc->grid;
    if (!valid_grid(&g)) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_create: invalid grid descriptor");
    if (desc->precision < 0 || desc->precision > 2) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_create: bad precision");
    if (desc->n_passive < 0 || desc->n_passive > OBGC_MAX_PASSIVE)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_create: n_passive outside 0..8");
    if (desc->negatives < OBGC_NEGATIVES_NONE || desc->negatives > OBGC_NEGATIVES_ZERO)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_create: bad negatives mode");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(OBGC_ERR_NO_DEVICE, "obgc_create: no CUDA device");
    obgc_ctx* c = new obgc_ctx();
    c->desc = *desc;
    std::memset(&c->fields, 0, sizeof(c->fields));
    c->prec = desc->precision;
    c->ts = c->prec == OBGC_PREC_F32 ? 4 : 8;
    c->tc = c->prec == OBGC_PREC_F64 ? 8 : 4;
    c->V = variant_of(desc->npd);
    // slot order: required BGC tracers, then carried T / S
    int32_t req[32];
    const int nreq = required_tracers(&desc->npd, req);
    c->NB = nreq;
    int nt = 0;
    for (int q = 0; q < nreq && nt < MAX_NT; q++) c->names[nt++] = req[q];
    bool hasT = false;
    for (int q = 0; q < nreq; q++) hasT |= req[q] == OBGC_T;
    if (desc->carry_T && !hasT && nt < MAX_NT) c->names[nt++] = OBGC_T;
    if (desc->carry_S && nt < MAX_NT) c->names[nt++] = OBGC_S;
    c->NT = nt;
    // passive slots after the main ones; a tendency source must be a carbonate tracer of the model
    c->NP = desc->n_passive;
    bool need_out[2] = {false, false};
    for (int p = 0; p < c->NP; p++) {
        const int src = desc->passive_tendency_of[p] - 1;
        bool carried = false;
        for (int q = 0; q < nreq; q++) carried |= req[q] == src;
        if (src != -1 && (!(src == OBGC_DIC || src == OBGC_ALK) || !carried)) {
            delete c;
            return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_create: a passive tracer's tendency source must be the model's DIC or Alk");
        }
        c->psrc[p] = src;
        if (src >= 0) need_out[src == OBGC_ALK] = true;
        c->names[c->NT + p] = OBGC_PASSIVE(p);
    }
    for (int r = c->NP; r > 0;) {   // launches of 4, 2 and 1 passive tracers
        const int n = r >= 4 ? 4 : r >= 2 ? 2 : 1;
        c->pchunk[c->nchunk++] = n;
        r -= n;
    }
    c->extent = g.stride_k * (int64_t)g.Nz;
    int rc = negatives_spec(desc->npd, desc->negatives, c->NT, c->names, desc->zero_exclude, desc->invalid_fill_value,
                            &c->neg);
    if (rc == OBGC_OK && c->NP > 0) {
        // ZeroNegativeTracers reaches every tracer of the model (negative_tracers.jl:23-29); the
        // ScaleNegativeTracers groups are named conserved tracers, none of them passive
        int pn[OBGC_MAX_PASSIVE];
        for (int p = 0; p < c->NP; p++) pn[p] = -1;
        rc = negatives_spec(desc->npd, desc->negatives == OBGC_NEGATIVES_ZERO ? OBGC_NEGATIVES_ZERO : OBGC_NEGATIVES_NONE,
                            c->NP, pn, desc->zero_exclude, desc->invalid_fill_value, &c->neg_passive);
    }
    auto alloc = [&](void** p, size_t bytes) {
        if (rc != OBGC_OK) return;
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMalloc");
    };
    // FP32 and mixed without passive tracers can stage tiles with the tensor-memory accelerator (from
    // FP32 padded copies of the state): the tendency arrays then use the padded layout
    const bool tma_capable = (c->prec == OBGC_PREC_F32 || c->prec == OBGC_PREC_MIXED) && c->NP == 0;
    if (tma_capable) {
        c->pad_sj = ((int64_t)g.Nx + 2 * TMA_HX + 3) / 4 * 4;
        c->pad_sk = c->pad_sj * (g.Ny + 2 * HALO);
    }
    const int64_t g_extent = std::max<int64_t>(c->extent, c->pad_sk * g.Nz);
    for (int t = 0; t < c->NT + c->NP; t++) {
        alloc(&c->scratch[t], c->ts * c->extent);
        alloc(&c->G[t], c->tc * g_extent);
    }
    for (int q = 0; q < 2; q++)
        if (need_out[q]) alloc(&c->bgc_out[q], c->tc * c->extent);
    // drift profiles of every slot (only non-zero ones are flagged)
    std::vector<double> prof((size_t)MAX_NT * (g.Nz + 1), 0.0);
    for (int t = 0; t < c->NT; t++) {
        double w0;
        if (desc->advection && drift_speed(&desc->npd, c->names[t], &w0) && w0 != 0.0) {
            drift_profile(w0, desc->npd.open_bottom, g.Nz, &prof[(size_t)t * (g.Nz + 1)]);
            c->drift_mask |= 1u << t;
        }
    }
    alloc(&c->drift, c->tc * prof.size());
    c->par_prefix_segs = (g.Nz + 1) / 2 - 1;
    if (c->par_prefix_segs > 0) alloc(&c->par_prefix, c->tc * 2 * (size_t)c->par_prefix_segs * g.Nx * g.Ny);
    alloc((void**)&c->d_time, sizeof(double));
    alloc((void**)&c->d_status, sizeof(int));
    if (rc == OBGC_OK) {
        cudaError_t e = cudaHostAlloc((void**)&c->h_status, sizeof(int), cudaHostAllocDefault);
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaHostAlloc(status)");
        else *c->h_status = 0;
    }
    c->n_partial = 4 * 152;
    alloc((void**)&c->partial, sizeof(DD) * c->n_partial);
    alloc((void**)&c->d_budget, sizeof(double));
    if (rc == OBGC_OK) {
        cudaError_t e;
        if (c->tc == 4) {
            std::vector<float> pf(prof.begin(), prof.end());
            e = cudaMemcpy(c->drift, pf.data(), 4 * pf.size(), cudaMemcpyHostToDevice);
        } else {
            e = cudaMemcpy(c->drift, prof.data(), 8 * prof.size(), cudaMemcpyHostToDevice);
        }
        if (e != cudaSuccess) rc = cuda_fail(e, "cudaMemcpy(drift)");
    }
    if (rc == OBGC_OK && (cudaEventCreate(&c->ev_begin) != cudaSuccess || cudaEventCreate(&c->ev_end) != cudaSuccess))
        rc = fail(OBGC_ERR_CUDA, "cudaEventCreate");
    if (rc == OBGC_OK && tma_capable) rc = setup_tma(c);
    if (rc == OBGC_OK && tma_capable &&
        (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
         cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
         cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess))
        rc = fail(OBGC_ERR_CUDA, "cudaStreamCreate / cudaEventCreate (pre-pass side stream)");
    // persistent grid size
    if (rc == OBGC_OK) {
        const FusedEntry* fe = c->V >= 0 ? find_fused(c->prec, c->V, c->NT) : nullptr;
        int dev = 0, nsm = 152, bps = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (fe) {
            int r2 = fe->occupancy(&bps);
            if (r2 != OBGC_OK) rc = r2;
        }
        c->blocks = nsm * (bps > 0 ? bps : 1);
        for (int q = 0; q < c->nchunk && rc == OBGC_OK; q++) {
            const int n = c->pchunk[q];
            const FusedEntry* pe = find_fused(c->prec, V_EXTERNAL, n);
            if (!pe) { rc = fail(OBGC_ERR_UNSUPPORTED, "obgc_create: no passive-tracer kernel for this precision"); break; }
            int pb = 1;
            rc = pe->occupancy(&pb);
            c->pblocks[n] = nsm * (pb > 0 ? pb : 1);
        }
    }
    if (rc != OBGC_OK) {
        ctx_free(c);
        return rc;
    }
    *out = c;
    return OBGC_OK;
}

extern "C" int obgc_destroy(obgc_ctx* ctx) { return ctx_free(ctx); }

extern "C" int obgc_bind_fields(obgc_ctx* c, const obgc_fields* f) {
    if (!c || !f) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_bind_fields: null argument");
    for (int t = 0; t < c->NT; t++) {
        void* p = f->tracers[c->names[t]];
        if (!p) return fail(OBGC_ERR_INVALID_ARGUMENT, std::string("obgc_bind_fields: missing tracer slot ") + std::to_string(c->names[t]));
        c->user[t] = p;
    }
    for (int p = 0; p < c->NP; p++) {
        if (!f->passive[p]) return fail(OBGC_ERR_INVALID_ARGUMENT, std::string("obgc_bind_fields: missing passive tracer ") + std::to_string(p));
        c->user[c->NT + p] = f->passive[p];
    }
    c->fields = *f;
    c->bound = true;
    c->bind_version++;
    // tensor maps of the bound arrays (the TMA-staged steps' first stage), when their layout allows
    // them: 16-byte aligned origins and row / level strides
    c->umaps_ok = false;
    if (c->tma_ready && c->tma_encode && c->prec == OBGC_PREC_F32) {
        const obgc_grid& g = c->desc.grid;
        bool ok = (g.stride_j * 4) % 16 == 0 && (g.stride_k * 4) % 16 == 0;
        for (int t = 0; t < c->NT && ok; t++) ok = reinterpret_cast<uintptr_t>(c->user[t]) % 16 == 0;
        if (ok) {
            auto encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(c->tma_encode);
            std::vector<CUtensorMap> maps(MAX_NT);
            std::memset(maps.data(), 0, sizeof(CUtensorMap) * maps.size());
            for (int t = 0; t < c->NT && ok; t++) {
                const cuuint64_t dims[3] = {(cuuint64_t)g.Nx, (cuuint64_t)g.Ny, (cuuint64_t)g.Nz};
                const cuuint64_t strides[2] = {(cuuint64_t)g.stride_j * sizeof(float), (cuuint64_t)g.stride_k * sizeof(float)};
                const cuuint32_t box[3] = {(cuuint32_t)TMA_TILE_W, (cuuint32_t)TILE_H, 1};
                const cuuint32_t es[3] = {1, 1, 1};
                ok = encode(&maps[t], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, c->user[t], dims, strides, box, es,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
            }
            if (ok) {
                const cudaError_t e = cudaMemcpy(c->d_tmaps + 2 * MAX_NT, maps.data(), sizeof(CUtensorMap) * MAX_NT,
                                                 cudaMemcpyHostToDevice);
                if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(tensor maps of the bound arrays)");
                c->umaps_ok = true;
            }
        }
    }
    return OBGC_OK;
}

extern "C" int obgc_set_profiling(obgc_ctx* c, int32_t on) {
    if (!c) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_profiling: null context");
    c->profile = on != 0;
    return OBGC_OK;
}

// slot of a tracer code (enum obgc_tracer or OBGC_PASSIVE(p)), or -1
static int slot_named(const obgc_ctx* c, int name) {
    for (int t = 0; t < c->NT + c->NP; t++)
        if (c->names[t] == name) return t;
    return -1;
}

extern "C" int obgc_set_gas_exchange_on(obgc_ctx* c, int32_t tracer, const obgc_gas_exchange* g, int32_t dic, int32_t alk) {
    if (!c || (g && !valid_gas(g))) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_gas_exchange_on: bad argument");
    const int target = slot_named(c, tracer);
    if (target < 0) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_gas_exchange_on: the model does not carry the tracer");
    obgc_ctx::GasCond* slot = nullptr;
    for (auto& gc : c->gas)
        if (gc.on && gc.target == target) slot = &gc;
    if (!g) {   // remove the tracer's condition
        if (slot) slot->on = false;
        c->bind_version++;
        return OBGC_OK;
    }
    const int sd = g->gas == OBGC_GAS_CO2 ? slot_named(c, dic) : -1, sa = g->gas == OBGC_GAS_CO2 ? slot_named(c, alk) : -1;
    if (slot_named(c, OBGC_T) < 0 || slot_named(c, OBGC_S) < 0 || (g->gas == OBGC_GAS_CO2 && (sd < 0 || sa < 0)))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_gas_exchange: the model does not carry the tracers this gas needs");
    for (auto& gc : c->gas)
        if (!slot && !gc.on) slot = &gc;
    if (!slot) return fail(OBGC_ERR_UNSUPPORTED, "obgc_set_gas_exchange_on: more than 4 gas exchange conditions");
    const size_t cols = (size_t)c->desc.grid.Nx * c->desc.grid.Ny;
    if (!slot->flux) OBGC_CUDA(cudaMalloc(&slot->flux, sizeof(double) * cols));
    // the warm start of the pCO2 solve: zero (none yet) whenever the condition is (re)set
    if (!slot->H) OBGC_CUDA(cudaMalloc(&slot->H, sizeof(double) * cols));
    OBGC_CUDA(cudaMemset(slot->H, 0, sizeof(double) * cols));
    slot->g = *g;
    slot->target = target;
    slot->dic = sd;
    slot->alk = sa;
    slot->on = true;
    c->bind_version++;   // a captured graph holds the previous flux setup
    return OBGC_OK;
}

extern "C" int obgc_set_gas_exchange(obgc_ctx* c, int32_t gas, const obgc_gas_exchange* g) {
    if (!c || (gas != OBGC_GAS_CO2 && gas != OBGC_GAS_O2) || (g && g->gas != gas))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_gas_exchange: bad argument");
    return obgc_set_gas_exchange_on(c, gas == OBGC_GAS_CO2 ? OBGC_DIC : OBGC_O2, g, OBGC_DIC, OBGC_ALK);
}

extern "C" int obgc_set_forcing(obgc_ctx* c, int32_t tracer, const void* rate, double t_start, double t_end) {
    if (!c || std::isnan(t_start) || std::isnan(t_end) || t_end < t_start)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_forcing: bad argument");
    const int t = slot_named(c, tracer);
    if (t < 0) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_forcing: the model does not carry the tracer");
    obgc_ctx::ForcingSpec* f = nullptr;
    for (auto& x : c->frc)
        if (x.rate && x.slot == t) f = &x;
    if (!rate) {
        if (f) *f = obgc_ctx::ForcingSpec();
        c->bind_version++;
        return OBGC_OK;
    }
    for (auto& x : c->frc)
        if (!f && !x.rate) f = &x;
    if (!f) return fail(OBGC_ERR_UNSUPPORTED, "obgc_set_forcing: more than 4 forced tracers");
    f->slot = t;
    f->rate = rate;
    f->t0 = t_start;
    f->t1 = t_end;
    c->bind_version++;
    return OBGC_OK;
}

extern "C" int obgc_set_diffusivity(obgc_ctx* c, double kappa_h, double kappa_z, const double* kappa_z_faces) {
    if (!c || !(kappa_h >= 0) || !(kappa_z >= 0)) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_diffusivity: bad argument");
    const obgc_grid& g = c->desc.grid;
    const int Nz = g.Nz;
    std::vector<double> k(Nz + 1, 0.0);
    bool any = false;
    const double idz2 = (double)Nz * Nz / (g.Lz * g.Lz);
    for (int f = 1; f < Nz; f++) {   // the bottom (0) and top (Nz) faces are walls
        const double kf = kappa_z_faces ? kappa_z_faces[f] : kappa_z;
        if (!(kf >= 0)) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_diffusivity: negative diffusivity");
        k[f] = kf * idz2;
        any = any || kf > 0;
    }
    if (c->kzz) { cudaFree(c->kzz); c->kzz = nullptr; }
    if (c->kzf) { cudaFree(c->kzf); c->kzf = nullptr; }
    if (any) {
        // the faces' kappa for the implicit form (the explicit form below carries kappa / dz^2)
        std::vector<double> kf(Nz + 1, 0.0);
        for (int f = 1; f < Nz; f++) kf[f] = kappa_z_faces ? kappa_z_faces[f] : kappa_z;
        OBGC_CUDA(cudaMalloc(&c->kzf, sizeof(double) * (Nz + 1)));
        OBGC_CUDA(cudaMemcpy(c->kzf, kf.data(), sizeof(double) * (Nz + 1), cudaMemcpyHostToDevice));
        if (!c->thomas) OBGC_CUDA(cudaMalloc(&c->thomas, sizeof(double) * 6 * Nz));
        OBGC_CUDA(cudaMalloc(&c->kzz, c->tc * (Nz + 1)));
        if (c->tc == 4) {
            std::vector<float> kf(k.begin(), k.end());
            OBGC_CUDA(cudaMemcpy(c->kzz, kf.data(), 4 * (Nz + 1), cudaMemcpyHostToDevice));
        } else {
            OBGC_CUDA(cudaMemcpy(c->kzz, k.data(), 8 * (Nz + 1), cudaMemcpyHostToDevice));
        }
    }
    c->kappa_h = kappa_h;
    c->bind_version++;
    return OBGC_OK;
}

extern "C" int obgc_set_vertical_time_discretization(obgc_ctx* c, int32_t discretization) {
    if (!c || (discretization != OBGC_EXPLICIT && discretization != OBGC_VERTICALLY_IMPLICIT))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_vertical_time_discretization: bad argument");
    c->vimplicit = discretization == OBGC_VERTICALLY_IMPLICIT;
    c->bind_version++;
    return OBGC_OK;
}

extern "C" int obgc_set_sediment(obgc_ctx* c, int32_t n_sinking, const int32_t* sinking_names, int32_t receiver_name,
                                 double a, double b, double k) {
    if (!c || n_sinking < 0 || (n_sinking > 0 && !sinking_names)) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_sediment: bad argument");
    if (n_sinking == 0) {   // no sediment
        c->sed_recv = -1;
        c->sed_mask = 0;
        c->bind_version++;
        return OBGC_OK;
    }
    c->mg_on = false;        // one sediment model at a time
    // the sediment couples to the main launch's slots (passive tracers neither sink nor receive)
    uint32_t mask = 0;
    for (int q = 0; q < n_sinking; q++) {
        const int t = slot_named(c, sinking_names[q]);
        if (t < 0 || t >= c->NT) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_sediment: a sinking tracer is not carried by the model");
        mask |= 1u << t;
    }
    const int r = slot_named(c, receiver_name);
    if (r < 0 || r >= c->NT) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_sediment: the receiver is not carried by the model");
    const size_t cols = (size_t)c->desc.grid.Nx * c->desc.grid.Ny;
    if (!c->sed_storage) {
        OBGC_CUDA(cudaMalloc(&c->sed_storage, c->ts * cols));
        OBGC_CUDA(cudaMemset(c->sed_storage, 0, c->ts * cols));
        OBGC_CUDA(cudaMalloc(&c->sed_G, c->tc * cols));
        OBGC_CUDA(cudaMemset(c->sed_G, 0, c->tc * cols));
    }
    c->sed_recv = r;
    c->sed_mask = mask;
    c->sed_a = a; c->sed_b = b; c->sed_k = k;
    c->bind_version++;
    return OBGC_OK;
}

extern "C" int obgc_multig_default_params(obgc_multig_params* p) {
    if (!p) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_multig_default_params: null argument");
    std::memset(p, 0, sizeof(*p));
    // SimpleMultiGSediment keyword defaults (simple_multi_G.jl:101-120)
    p->fast_decay_rate = 2.0 / 86400.0;
    p->slow_decay_rate = 0.2 / 86400.0;
    p->fast_redfield = 0.1509;
    p->slow_redfield = 0.13;
    p->fast_fraction = 0.74;
    p->slow_fraction = 0.26;
    p->refactory_fraction = 0.1;
    p->sedimentation_rate = 0.0;          // from the grid at obgc_set_multig_sediment
    p->anoxia_half_saturation = 1.0;
    p->sinking_redfield = 6.56;
    const double nox[6] = {-1.9785, 0.2261, -0.0615, -0.0289, -0.36109, -0.0232};
    const double den[6] = {-3.0790, 1.7509, 0.0593, -0.1923, 0.0604, 0.0662};
    const double anx[6] = {-3.9476, 2.6269, -0.2426, -1.3349, 0.1826, -0.0143};
    std::memcpy(p->nitrate_oxidation, nox, sizeof(nox));
    std::memcpy(p->denitrification, den, sizeof(den));
    std::memcpy(p->anoxic, anx, sizeof(anx));
    return OBGC_OK;
}

extern "C" int obgc_set_multig_sediment(obgc_ctx* c, const obgc_multig_params* p, int32_t n_sinking,
                                        const int32_t* sinking_names) {
    if (!c || n_sinking < 0 || n_sinking > 4 || (n_sinking > 0 && (!sinking_names || !p)))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_multig_sediment: bad argument");
    if (n_sinking == 0) {
        c->mg_on = false;
        c->bind_version++;
        return OBGC_OK;
    }
    const obgc_grid& g = c->desc.grid;
    const int no3 = slot_named(c, OBGC_NO3), nh4 = slot_named(c, OBGC_NH4), o2 = slot_named(c, OBGC_O2);
    if (no3 < 0 || nh4 < 0 || o2 < 0 || no3 >= c->NT || nh4 >= c->NT || o2 >= c->NT)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_multig_sediment: the model needs NO3, NH4 and O2 (LOBSTER with Oxygen)");
    obgc_multig_params q = *p;
    if (!(q.sedimentation_rate > 0)) {
        // 982 |znode(1, 1, 1)|^-1.548 cm/year: the depth of the bottom cell's centre
        const double zb = -g.Lz + 0.5 * g.Lz / g.Nz;
        q.sedimentation_rate = 982.0 * std::pow(std::fabs(zb), -1.548);
    }
    for (int s = 0; s < n_sinking; s++) {
        const int t = slot_named(c, sinking_names[s]);
        double w0 = 0.0;
        if (t < 0 || t >= c->NT || !drift_speed(&c->desc.npd, sinking_names[s], &w0))
            return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_multig_sediment: a sinking tracer is not a sinking tracer of the model");
        std::vector<double> prof((size_t)g.Nz + 1);
        drift_profile(w0, c->desc.npd.open_bottom, g.Nz, prof.data());
        c->mg_sink[s] = t;
        c->mg_w0[s] = c->desc.advection ? prof[0] : 0.0;
    }
    const size_t cols = (size_t)g.Nx * g.Ny;
    if (!c->mg_state) {
        OBGC_CUDA(cudaMalloc(&c->mg_state, sizeof(double) * 4 * cols));
        OBGC_CUDA(cudaMemset(c->mg_state, 0, sizeof(double) * 4 * cols));
        OBGC_CUDA(cudaMalloc(&c->mg_gcache, sizeof(double) * 3 * cols));
        OBGC_CUDA(cudaMemset(c->mg_gcache, 0, sizeof(double) * 3 * cols));
        OBGC_CUDA(cudaMalloc(&c->mg_flux, sizeof(double) * 3 * cols));
        OBGC_CUDA(cudaMemset(c->mg_flux, 0, sizeof(double) * 3 * cols));
    }
    c->mg = make_multig(q);
    c->mg_nsink = n_sinking;
    c->mg_no3 = no3; c->mg_nh4 = nh4; c->mg_o2 = o2;
    c->mg_on = true;
    c->sed_recv = -1;        // one sediment model at a time
    c->sed_mask = 0;
    c->bind_version++;
    return OBGC_OK;
}

extern "C" int obgc_multig_sediment_state(obgc_ctx* c, const double* set, double* get) {
    if (!c || !c->mg_state) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_multig_sediment_state: no SimpleMultiG sediment");
    const size_t cols = (size_t)c->desc.grid.Nx * c->desc.grid.Ny;
    OBGC_CUDA(cudaDeviceSynchronize());
    if (set) {
        OBGC_CUDA(cudaMemcpy(c->mg_state, set, sizeof(double) * 3 * cols, cudaMemcpyHostToDevice));
        OBGC_CUDA(cudaMemset(c->mg_state + 3 * cols, 0, sizeof(double) * cols));   // the clock restarts
    }
    if (get) OBGC_CUDA(cudaMemcpy(get, c->mg_state, sizeof(double) * 3 * cols, cudaMemcpyDeviceToHost));
    return OBGC_OK;
}

extern "C" int obgc_sediment_storage(obgc_ctx* c, const double* set, double* get) {
    if (!c || !c->sed_storage) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_sediment_storage: no sediment");
    const size_t cols = (size_t)c->desc.grid.Nx * c->desc.grid.Ny;
    OBGC_CUDA(cudaDeviceSynchronize());
    if (set) {
        if (c->ts == 4) {
            std::vector<float> h(set, set + cols);
            OBGC_CUDA(cudaMemcpy(c->sed_storage, h.data(), 4 * cols, cudaMemcpyHostToDevice));
        } else {
            OBGC_CUDA(cudaMemcpy(c->sed_storage, set, 8 * cols, cudaMemcpyHostToDevice));
        }
    }
    if (get) {
        if (c->ts == 4) {
            std::vector<float> h(cols);
            OBGC_CUDA(cudaMemcpy(h.data(), c->sed_storage, 4 * cols, cudaMemcpyDeviceToHost));
            for (size_t q = 0; q < cols; q++) get[q] = h[q];
        } else {
            OBGC_CUDA(cudaMemcpy(get, c->sed_storage, 8 * cols, cudaMemcpyDeviceToHost));
        }
    }
    return OBGC_OK;
}

extern "C" int obgc_set_tiling(obgc_ctx* c, int32_t TZ) {
    if (!c || TZ < 1) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_tiling: bad argument");
    c->TZ = TZ;
    c->graph_version = ~0ull;
    return OBGC_OK;
}

extern "C" int obgc_update_state(obgc_ctx* c, double t, void* stream) {
    if (!c || !c->bound) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_update_state: context not bound");
    if (!c->fields.PAR) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_update_state: no PAR field bound");
    if (c->neg.mode != OBGC_NEGATIVES_NONE) {
        // update_biogeochemical_state! runs the modifiers before the light (src/OceanBioME.jl:161-167)
        void* f[MAX_NT];
        for (int t = 0; t < c->NT; t++) f[t] = c->user[t];
        int rc = launch_negatives(c->neg, c->ts, f, c->desc.grid, static_cast<cudaStream_t>(stream));
        if (rc == OBGC_OK && c->neg_passive.mode != OBGC_NEGATIVES_NONE)
            rc = launch_negatives(c->neg_passive, c->ts, &c->user[c->NT], c->desc.grid, static_cast<cudaStream_t>(stream));
        if (rc != OBGC_OK) return rc;
    }
    const void* P = c->fields.tracers[OBGC_P];
    return obgc_twoband_par(&c->desc.light, &c->desc.surface, &c->desc.grid, c->ts == 4 ? OBGC_F32 : OBGC_F64, P,
                            c->fields.PAR, t, stream);
}

extern "C" int obgc_compute_tendencies(obgc_ctx* c, double t, void* stream) {
    if (!c || !c->bound) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_compute_tendencies: context not bound");
    if (!c->fields.PAR) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_compute_tendencies: no PAR field bound");
    return obgc_npd_tendencies(&c->desc.npd, &c->desc.grid, c->ts == 4 ? OBGC_F32 : OBGC_F64,
                               (const void* const*)c->fields.tracers, c->fields.PAR, c->fields.G, t, stream);
}

template <typename TS, typename TC>
static void fill_args(obgc_ctx* c, SubstepArgs<TS, TC>& a) {
    const obgc_grid& g = c->desc.grid;
    std::memset(&a, 0, sizeof(a));
    a.Nx = g.Nx; a.Ny = g.Ny; a.Nz = g.Nz;
    a.periodic_x = g.topology_x == OBGC_PERIODIC;
    a.periodic_y = g.topology_y == OBGC_PERIODIC;
    a.flat_x = g.topology_x == OBGC_FLAT || !c->desc.advection;
    a.flat_y = g.topology_y == OBGC_FLAT || !c->desc.advection;
    a.sj = g.stride_j; a.sk = g.stride_k;
    a.osj = g.stride_j; a.osk = g.stride_k;
    a.vsj = g.stride_j; a.vsk = g.stride_k;
    a.gsj = g.stride_j; a.gsk = g.stride_k;
    a.out_halo = 0;
    a.tma_layout = 0;
    a.tmap = nullptr;
    a.tma_x0 = a.tma_y0 = 0;
    a.dx = TC(g.Lx / g.Nx); a.dy = TC(g.Ly / g.Ny); a.dz = TC(g.Lz / g.Nz); a.Lz = TC(g.Lz);
    a.inv_dx = TC(g.Nx / g.Lx); a.inv_dy = TC(g.Ny / g.Ly); a.inv_dz = TC(g.Nz / g.Lz);
    if (c->TZ > 0) {
        a.TZ = c->TZ < g.Nz ? c->TZ : g.Nz;
    } else {
        // 8 levels per item (best at 256x256x64), fewer when the grid has too few tiles to fill the
        // GPU: a 160x32 2-D grid has 5 tiles, and 2-level items gave it the shortest step
        const int tiles = ((g.Nx + STEP_BX - 1) / STEP_BX) * ((g.Ny + STEP_BY - 1) / STEP_BY);
        int tz = 8;
        while (tz > 2 && (int64_t)tiles * ((g.Nz + tz - 1) / tz) < c->blocks) tz /= 2;
        a.TZ = tz < g.Nz ? tz : g.Nz;
    }
    a.nseg = (g.Nz + a.TZ - 1) / a.TZ;
    a.ntx = (g.Nx + STEP_BX - 1) / STEP_BX;
    a.nty = (g.Ny + STEP_BY - 1) / STEP_BY;
    a.n_items = a.ntx * a.nty * a.nseg;
    for (int t = 0; t < c->NT; t++) a.G[t] = (TC*)c->G[t];
    a.u = c->desc.advection ? (const TS*)c->fields.u : nullptr;
    a.v = c->desc.advection ? (const TS*)c->fields.v : nullptr;
    a.w = c->desc.advection ? (const TS*)c->fields.w : nullptr;
    a.drift = (const TC*)c->drift;
    a.drift_mask = c->drift_mask;
    a.bgc = make_params<TC>(c->desc.npd);
    a.light = make_twoband<TC>(c->desc.light);
    a.surf_kind = c->desc.surface.kind;
    a.surf_value = TC(c->desc.surface.value);
    a.surf_field = (const TS*)c->desc.surface.field;
    a.d_time = c->d_time;
    a.status = c->d_status;
    a.neg = c->neg;        // the modifier after every substep, fused into the substep's update
    a.kh_dx = g.topology_x == OBGC_FLAT ? TC(0) : TC(c->kappa_h * g.Nx / g.Lx);
    a.kh_dy = g.topology_y == OBGC_FLAT ? TC(0) : TC(c->kappa_h * g.Ny / g.Ly);
    a.kzz = c->vimplicit ? nullptr : (const TC*)c->kzz;   // the implicit form leaves the vertical part out
    a.sed_recv1 = c->sed_recv >= 0 ? c->sed_recv + 1 : 0;
    a.sed_sink_mask = c->sed_mask;
    a.sed_a = TC(c->sed_a); a.sed_b = TC(c->sed_b); a.sed_k = TC(c->sed_k);
    a.sed_storage = (TS*)c->sed_storage;
    a.sed_G = (TC*)c->sed_G;
    if (c->mg_on) {
        const int64_t cols = (int64_t)g.Nx * g.Ny;
        const int slots[3] = {c->mg_no3, c->mg_nh4, c->mg_o2};
        for (int q = 0; q < 3; q++) {
            a.bot_slot1[q] = slots[q] + 1;
            a.bot_flux[q] = c->mg_flux + q * cols;
        }
    }
}

// Whether the device clock (d_time) must advance with the steps: the default surface PAR and the
// forcing windows read it.
static bool needs_clock(const obgc_ctx* c) {
    bool f = false;
    for (const auto& x : c->frc) f = f || x.rate != nullptr;
    return c->desc.surface.kind == OBGC_SURFACE_PAR_DEFAULT || f;
}

// The surface-flux and forcing slots of the launch over slots [b, b + n).
// The TwoBand chlorophyll sums above every segment of the stage's input, for the substep launch that
// follows (segments of two levels or more, a model with the in-kernel PAR); otherwise the work items
// sum them themselves.
template <typename TS, typename TC>
static int launch_par_prefix(obgc_ctx* c, SubstepArgs<TS, TC>& a, cudaStream_t st) {
    a.par_prefix = nullptr;
    c->prefix_on = false;
    if (!c->par_prefix || c->V == V_EXTERNAL || a.nseg < 2 || a.nseg - 1 > c->par_prefix_segs) return OBGC_OK;
    const int64_t cols = (int64_t)a.Nx * a.Ny;
    par_prefix_kernel<TS, TC><<<(unsigned)((cols + PP_COLS - 1) / PP_COLS), 256, 0, st>>>(
        a.in[slot_of_P(c->V)], a.sj, a.sk, a.Nx, a.Ny, a.Nz, a.TZ, a.nseg, a.light, (TC*)c->par_prefix);
    OBGC_LAUNCHED("par_prefix_kernel");
    a.par_prefix = (const TC*)c->par_prefix;
    c->prefix_on = true;
    return OBGC_OK;
}

// The window slots' vertical face fluxes of the stage's input, for the TMA-staged substep launch that
// follows (when the model has sinking tracers in the window slots).
template <typename TS, typename TC>
static int launch_sink_flux(obgc_ctx* c, SubstepArgs<TS, TC>& a, cudaStream_t st) {
    a.fz_pre = nullptr;
    c->sinkpre_on = false;
    const int wa = window_a(c->V), wb = window_b(c->V);
    if (!(a.drift_mask & ((1u << wa) | (1u << wb)))) return OBGC_OK;
    if (!c->fz_pre) return fail(OBGC_ERR_UNSUPPORTED, "obgc_step: no buffer for the sinking fluxes");
    const int64_t cols = (int64_t)a.Nx * a.Ny;
    const dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((a.Nz + 1 + 8 * SF_FACES - 1) / (8 * SF_FACES)));
    sink_flux_kernel<TS, TC><<<grid, 256, 0, st>>>(a.in[wa], a.in[wb], a.sj, a.sk, a.Nx, a.Ny, a.Nz, a.drift, wa, wb,
                                                   (TC*)c->fz_pre);
    OBGC_LAUNCHED("sink_flux_kernel");
    a.fz_pre = (const TC*)c->fz_pre;
    c->sinkpre_on = true;
    return OBGC_OK;
}

template <typename TS, typename TC>
static void launch_terms(const obgc_ctx* c, SubstepArgs<TS, TC>& a, int b, int n) {
    int nt = 0, nf = 0;
    for (int q = 0; q < MAX_TOP; q++) { a.top_slot1[q] = 0; a.top_flux[q] = nullptr; }
    for (const auto& gc : c->gas)
        if (gc.on && gc.target >= b && gc.target < b + n && nt < MAX_TOP) {
            a.top_slot1[nt] = gc.target - b + 1;
            a.top_flux[nt++] = gc.flux;
        }
    for (int q = 0; q < MAX_FRC; q++) { a.frc_slot1[q] = 0; a.frc[q] = nullptr; }
    for (const auto& f : c->frc)
        if (f.rate && f.slot >= b && f.slot < b + n && nf < MAX_FRC) {
            a.frc_slot1[nf] = f.slot - b + 1;
            a.frc[nf] = (const TS*)f.rate;
            a.frc_t0[nf] = f.t0;
            a.frc_t1[nf++] = f.t1;
        }
}

// The SimpleMultiG sediment's per-column kernel on the state in `cur` (dt = 0: the coupled
// tendencies only).
template <typename TS>
static int launch_multig(obgc_ctx* c, void* const* cur, double dt, cudaStream_t st) {
    if (!c->mg_on) return OBGC_OK;
    const obgc_grid& g = c->desc.grid;
    MultiGArgs<TS> a;
    std::memset(&a, 0, sizeof(a));
    a.m = c->mg;
    a.Nx = g.Nx; a.Ny = g.Ny; a.sj = g.stride_j;
    a.n_sink = c->mg_nsink;
    for (int q = 0; q < c->mg_nsink; q++) { a.sink[q] = (const TS*)cur[c->mg_sink[q]]; a.w0[q] = c->mg_w0[q]; }
    a.no3 = (const TS*)cur[c->mg_no3];
    a.nh4 = (const TS*)cur[c->mg_nh4];
    a.o2 = (const TS*)cur[c->mg_o2];
    a.state = c->mg_state;
    a.gcache = c->mg_gcache;
    a.flux = c->mg_flux;
    a.dt = dt;
    const int64_t cols = (int64_t)g.Nx * g.Ny;
    multig_kernel<TS><<<(unsigned)((cols + 127) / 128), 128, 0, st>>>(a);
    OBGC_LAUNCHED("multig_kernel");
    return OBGC_OK;
}

// Launch arguments of a context's steps of size dt: the main launch (a) and the passive launches
// (ap: no drift, no sediment, ZeroNegativeTracers only).
template <typename TS, typename TC>
struct StepPlan {
    SubstepArgs<TS, TC> a, ap;
    const FusedEntry* fe = nullptr;
    const FusedEntry* pe[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    bool impl = false;        // VerticallyImplicitTimeDiscretization with a vertical diffusivity
    double inv_dz2 = 0.0;
    int blocks = 0;
};

template <typename TS, typename TC>
static int plan_steps(obgc_ctx* c, const FusedEntry* fe, double dt, StepPlan<TS, TC>& p) {
    SubstepArgs<TS, TC>& a = p.a;
    fill_args<TS, TC>(c, a);
    a.dt_d = dt;
    a.dt = TC(dt);
    a.bgc_out[0] = (TC*)c->bgc_out[0];
    a.bgc_out[1] = (TC*)c->bgc_out[1];
    p.ap = a;
    p.ap.drift_mask = 0;
    p.ap.sed_recv1 = 0;
    for (int q = 0; q < 3; q++) { p.ap.bot_slot1[q] = 0; p.ap.bot_flux[q] = nullptr; }
    p.ap.sed_sink_mask = 0;
    p.ap.bgc_out[0] = p.ap.bgc_out[1] = nullptr;
    p.fe = fe;
    for (int q = 0; q < c->nchunk; q++) {
        p.pe[c->pchunk[q]] = find_fused(c->prec, V_EXTERNAL, c->pchunk[q]);
        if (!p.pe[c->pchunk[q]]) return fail(OBGC_ERR_UNSUPPORTED, "obgc_step: no passive-tracer kernel for this precision");
    }
    // VerticallyImplicitTimeDiscretization: after every stage an implicit solve of every column and
    // slot, followed by the negative-tracer modifier (which the substep then must not fuse: it acts
    // on the diffused state)
    const obgc_grid& gz = c->desc.grid;
    p.impl = c->vimplicit && c->kzf;
    p.inv_dz2 = (double)gz.Nz * gz.Nz / (gz.Lz * gz.Lz);
    if (p.impl) a.neg.mode = OBGC_NEGATIVES_NONE;
    p.blocks = c->blocks < a.n_items ? c->blocks : a.n_items;
    return OBGC_OK;
}

// The Thomas factors of the implicit vertical diffusion for steps of this dt (when it is on).
template <typename TS, typename TC>
static int launch_thomas(obgc_ctx* c, const StepPlan<TS, TC>& p, double dt, cudaStream_t st) {
    if (!p.impl) return OBGC_OK;
    thomas_factors_kernel<<<1, 32, 0, st>>>(c->kzf, c->desc.grid.Nz, p.inv_dz2, dt, c->thomas);
    OBGC_LAUNCHED("thomas_factors_kernel");
    return OBGC_OK;
}

// RK3 stage `stg` from the slot arrays cur[] into nxt[]: the gas-exchange flux of every condition,
// the main launch (the model's tracers, T and S), the passive launches (their BGC tendency, if any,
// is the main launch's DIC / Alk tendency of the same stage), then the implicit vertical solve.
template <typename TS, typename TC>
static int enqueue_stage(obgc_ctx* c, StepPlan<TS, TC>& p, int stg, void* const* cur, void* const* nxt, cudaStream_t st,
                         bool profile, size_t& ev) {
    SubstepArgs<TS, TC>& a = p.a;
    SubstepArgs<TS, TC>& ap = p.ap;
    const int NS = c->NT + c->NP;
    const obgc_grid& grid = c->desc.grid;
    // every gas-exchange condition in one launch (CO2 conditions with the first one's
    // carbon-chemistry options share the column's T/S constants)
    {
        GasMulti gm;
        std::memset(&gm, 0, sizeof(gm));
        gm.status = c->d_status;
        const obgc_carbon_options* first = nullptr;
        for (const auto& gc : c->gas) {
            if (!gc.on) continue;
            const int q = gm.n++;
            gm.g[q] = gc.g;
            gm.flux[q] = gc.flux;
            gm.H[q] = gc.H;
            if (gc.g.gas == OBGC_GAS_CO2) {
                gm.DIC[q] = cur[gc.dic];
                gm.Alk[q] = cur[gc.alk];
                if (!first) first = &gc.g.carbon;
                gm.share[q] = std::memcmp(first, &gc.g.carbon, sizeof(obgc_carbon_options)) == 0;
            } else {
                gm.O2[q] = cur[gc.target];
            }
        }
        if (gm.n > 0) {
            const int rg = launch_gas_exchange_multi<TS>(gm, &grid, cur[slot_named(c, OBGC_T)], cur[slot_named(c, OBGC_S)], st);
            if (rg != OBGC_OK) return rg;
        }
    }
    for (SubstepArgs<TS, TC>* x : {&a, &ap}) {
        x->first_stage = stg == 0;
        x->write_G = stg < 2;
        x->gamma = TC(rk3_gamma(stg));
        x->zeta = TC(rk3_zeta(stg));
        x->c_stage = rk3_c(stg);
    }
    for (int t = 0; t < c->NT; t++) { a.in[t] = (const TS*)cur[t]; a.out[t] = (TS*)nxt[t]; }
    launch_terms(c, a, 0, c->NT);
    int rc = launch_par_prefix(c, a, st);
    if (rc != OBGC_OK) return rc;
    if (profile) OBGC_CUDA(cudaEventRecord(c->prof_events[ev++], st));
    rc = p.fe->launch(&a, p.blocks, st);
    if (rc != OBGC_OK) return rc;
    for (int q = 0, b = c->NT; q < c->nchunk; b += c->pchunk[q++]) {
        const int n = c->pchunk[q];
        for (int t = 0; t < MAX_NT; t++) { ap.in[t] = nullptr; ap.out[t] = nullptr; ap.G[t] = nullptr; ap.ext[t] = nullptr; }
        for (int t = 0; t < n; t++) {
            ap.in[t] = (const TS*)cur[b + t];
            ap.out[t] = (TS*)nxt[b + t];
            ap.G[t] = (TC*)c->G[b + t];
            const int src = c->psrc[b + t - c->NT];
            ap.ext[t] = src < 0 ? nullptr : (const TC*)c->bgc_out[src == OBGC_ALK];
        }
        ap.n_ext = n;
        ap.neg = c->neg_passive;
        if (p.impl) ap.neg.mode = OBGC_NEGATIVES_NONE;
        if (ap.neg.mode != OBGC_NEGATIVES_NONE) {
            ap.neg.nt = n;
            ap.neg.zero_skip = (c->neg_passive.zero_skip >> (b - c->NT)) & ((1u << n) - 1u);
        }
        launch_terms(c, ap, b, n);
        const int pb = c->pblocks[n] < ap.n_items ? c->pblocks[n] : ap.n_items;
        rc = p.pe[n]->launch(&ap, pb, st);
        if (rc != OBGC_OK) return rc;
    }
    if (p.impl) {
        const obgc_grid& gz = grid;
        ImplicitFields<TS> F;
        for (int t = 0; t < NS; t++) F.f[t] = (TS*)nxt[t];
        const int64_t nthr = (int64_t)gz.Nx * gz.Ny * NS;
        implicit_vertical_kernel<TS><<<(unsigned)((nthr + 127) / 128), 128, 0, st>>>(
            F, NS, gz.Nx, gz.Ny, gz.Nz, gz.stride_j, gz.stride_k, c->kzf, p.inv_dz2, a.dt_d, stg, c->thomas);
        OBGC_LAUNCHED("implicit_vertical_kernel");
        if (c->neg.mode != OBGC_NEGATIVES_NONE) {
            rc = launch_negatives(c->neg, sizeof(TS), const_cast<void**>(nxt), grid, st);
            if (rc == OBGC_OK && c->neg_passive.mode != OBGC_NEGATIVES_NONE)
                rc = launch_negatives(c->neg_passive, sizeof(TS), const_cast<void**>(nxt) + c->NT, grid, st);
            if (rc != OBGC_OK) return rc;
        }
    }
    if (profile) OBGC_CUDA(cudaEventRecord(c->prof_events[ev++], st));
    return OBGC_OK;
}

// The two pre-passes of a TMA-staged stage: the chlorophyll sums on the context's side stream (forked
// from and joined back into st by events, so it works eagerly and under stream capture) beside the
// sinking fluxes on st.
template <typename TS, typename TC>
static int launch_pre_passes(obgc_ctx* c, SubstepArgs<TS, TC>& a, cudaStream_t st) {
    if (!c->side) {
        int rc = launch_par_prefix(c, a, st);
        return rc == OBGC_OK ? launch_sink_flux(c, a, st) : rc;
    }
    OBGC_CUDA(cudaEventRecord(c->ev_fork, st));
    OBGC_CUDA(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
    int rc = launch_par_prefix(c, a, c->side);
    const cudaError_t e = cudaEventRecord(c->ev_join, c->side);   // joined even when the launch failed
    if (rc == OBGC_OK) rc = launch_sink_flux(c, a, st);
    const cudaError_t w = cudaStreamWaitEvent(st, c->ev_join, 0);
    if (rc != OBGC_OK) return rc;
    if (e != cudaSuccess) return cuda_fail(e, "cudaEventRecord(pre-pass join)");
    if (w != cudaSuccess) return cuda_fail(w, "cudaStreamWaitEvent(pre-pass join)");
    return OBGC_OK;
}

// Whether the steps can stage tiles with the tensor-memory accelerator: FP32 arithmetic (FP32 or
// mixed), the lean kernel (no closure, surface flux, forcing, fused modifier, sediment or replicate
// outputs), no passive tracers, no model w, no implicit vertical solve, and at least 8 cells in a
// periodic x and 6 in a periodic y.  The mixed path updates its FP64 state in place, so its stages
// must read no other cell of it: no sinking tracer outside the two flux pre-pass slots, and the
// chlorophyll sums from the pre-pass (or a single segment per column).
template <typename TS, typename TC>
static bool tma_eligible(obgc_ctx* c, const StepPlan<TS, TC>& p) {
    if (sizeof(TC) != 4 || !c->tma_ready || c->staging != 1 || c->NP != 0 || p.impl || p.a.w) return false;
    if (sizeof(TS) != sizeof(TC)) {
        const uint32_t slots = (1u << window_a(c->V)) | (1u << window_b(c->V));
        if ((p.a.drift_mask & ~slots) != 0u) return false;
        if (p.a.nseg > 1 && (!c->par_prefix || c->V == V_EXTERNAL || p.a.nseg - 1 > c->par_prefix_segs)) return false;
    }
    // a cell writes one periodic image per direction into the padded halos: a periodic direction needs
    // at least two halos' width of cells (8 in x, 6 in y)
    if ((p.a.periodic_x && p.a.Nx < 2 * TMA_HX) || (p.a.periodic_y && p.a.Ny < 2 * HALO)) return false;
    SubstepArgs<TS, TC> x = p.a;
    launch_terms(c, x, 0, c->NT);
    return !substep_needs_ext(x);
}

// Steps with TMA-staged tiles (the MODE 2 kernel: one tensor copy per tracer and level).  The caller's
// arrays are first copied into padded set 1 with their periodic images (pad_copy_kernel), then the
// 3 nsteps stages of the call run padded set 1 -> padded set 0 -> padded set 1 -> ... -> bound
// arrays: every stage but the last writes a padded set together with its periodic halo images, and
// only the last writes the caller's arrays.  When no tile needs the periodic wrap (and the caller's
// arrays have tensor maps) there is no copy: the first stage copies its tiles from them directly.
// Mixed precision: the FP64 bound arrays are updated in place by every stage, and the padded sets
// hold their FP32 rounding (the copy rounds them, each stage but the last writes the next set).
template <typename TS, typename TC>
static int enqueue_steps_tma(obgc_ctx* c, StepPlan<TS, TC>& p, double dt, int nsteps, cudaStream_t st, bool profile) {
    SubstepArgs<TS, TC>& a = p.a;
    const obgc_grid& g = c->desc.grid;
    const int64_t org = TMA_HX + (int64_t)HALO * c->pad_sj;   // the padded arrays' first interior cell
    launch_terms(c, a, 0, c->NT);
    a.gsj = c->pad_sj;
    a.gsk = c->pad_sk;
    const bool clock = needs_clock(c);
    size_t ev = 0;
    const int last = 3 * nsteps - 1;
    constexpr bool mixed = sizeof(TS) != sizeof(TC);
    bool none_wrap = !mixed && c->umaps_ok;
    for (int tj = 0; tj < a.nty && none_wrap; tj++)
        for (int ti = 0; ti < a.ntx && none_wrap; ti++) none_wrap = !tile_wraps(a, ti * STEP_BX, tj * STEP_BY);
    const bool copy_first = !none_wrap;
    // FP32 with tensor maps of the caller's arrays: only the wrapping tiles' boxes are copied, and the
    // first stage copies the other tiles from the caller's arrays
    const bool bands = copy_first && !mixed && c->umaps_ok;
    c->copied_first = copy_first;
    if (copy_first) {
        PadCopyArgs<TS> pc;
        std::memset(&pc, 0, sizeof(pc));
        pc.nt = c->NT;
        for (int t = 0; t < c->NT; t++) {
            pc.src[t] = (const TS*)c->user[t];
            pc.dst[t] = (float*)c->pad[1][t];
        }
        const int64_t n = (int64_t)(g.Nx + 2 * TMA_HX) * (g.Ny + 2 * HALO) * g.Nz;
        pad_copy_kernel<TS><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(pc, g.Nx, g.Ny, g.Nz, g.stride_j, g.stride_k, c->pad_sj,
                                                                     c->pad_sk, a.periodic_x, a.periodic_y, bands ? 1 : 0);
        OBGC_LAUNCHED("pad_copy_kernel");
    }
    for (int s = 0; s < nsteps; s++) {
        for (int stg = 0; stg < 3; stg++) {
            const int q = 3 * s + stg;          // the stage's place in the call
            a.first_stage = stg == 0;
            a.write_G = stg < 2;
            a.gamma = TC(rk3_gamma(stg));
            a.zeta = TC(rk3_zeta(stg));
            a.c_stage = rk3_c(stg);
            const bool from_user = q == 0 && (!copy_first || bands);   // this stage reads the caller's arrays
            const int pin = q == 0 ? 1 : (q - 1) % 2;       // else the padded set it reads
            if constexpr (mixed) {
                for (int t = 0; t < c->NT; t++) {
                    a.in[t] = (const TS*)c->user[t];
                    a.out[t] = (TS*)c->user[t];
                    a.pout[t] = q == last ? nullptr : (TC*)c->pad[q % 2][t] + org;
                }
                a.sj = a.osj = g.stride_j;
                a.sk = a.osk = g.stride_k;
                a.psj = c->pad_sj;
                a.psk = c->pad_sk;
            } else {
                for (int t = 0; t < c->NT; t++) {
                    a.in[t] = from_user ? (const TS*)c->user[t] : (const TS*)c->pad[pin][t] + org;
                    a.out[t] = q == last ? (TS*)c->user[t] : (TS*)c->pad[q % 2][t] + org;
                }
                a.sj = from_user ? g.stride_j : c->pad_sj;
                a.sk = from_user ? g.stride_k : c->pad_sk;
                a.osj = q == last ? g.stride_j : c->pad_sj;
                a.osk = q == last ? g.stride_k : c->pad_sk;
            }
            a.out_halo = q != last;
            a.tma_layout = 2;
            a.tmap = from_user ? c->d_tmaps + 2 * MAX_NT : c->d_tmaps + (size_t)pin * MAX_NT;
            a.tmap_wrap = q == 0 && bands ? c->d_tmaps + (size_t)1 * MAX_NT : nullptr;   // padded set 1
            a.tma_x0 = from_user ? -TMA_HX : 0;
            a.tma_y0 = from_user ? -HALO : 0;
            int rc = launch_pre_passes(c, a, st);
            if (rc != OBGC_OK) return rc;
            if (profile) OBGC_CUDA(cudaEventRecord(c->prof_events[ev++], st));
            rc = p.fe->launch(&a, p.blocks, st);
            if (rc != OBGC_OK) return rc;
            if (profile) OBGC_CUDA(cudaEventRecord(c->prof_events[ev++], st));
        }
        if (clock) {
            advance_time_kernel<<<1, 1, 0, st>>>(c->d_time, dt);
            OBGC_LAUNCHED("advance_time_kernel");
        }
    }
    return OBGC_OK;
}

// Enqueue nsteps steps on stream st (no synchronisation).  The state ping-pongs between the bound
// arrays and the context's scratch buffers; after an odd number of substeps the interior is copied
// back so the bound arrays always hold the result.
template <typename TS, typename TC>
static int enqueue_steps(obgc_ctx* c, const FusedEntry* fe, double dt, int nsteps, cudaStream_t st, bool profile) {
    StepPlan<TS, TC> p;
    int rc = plan_steps<TS, TC>(c, fe, dt, p);
    if (rc != OBGC_OK) return rc;
    c->last_used_tma = tma_eligible<TS, TC>(c, p);
    if (c->last_used_tma) return enqueue_steps_tma<TS, TC>(c, p, dt, nsteps, st, profile);
    const int NS = c->NT + c->NP;
    void* cur[MAX_NT];
    void* nxt[MAX_NT];
    for (int t = 0; t < NS; t++) { cur[t] = c->user[t]; nxt[t] = c->scratch[t]; }
    const bool clock = needs_clock(c);
    rc = launch_thomas<TS, TC>(c, p, dt, st);
    if (rc != OBGC_OK) return rc;
    size_t ev = 0;
    const obgc_grid& grid = c->desc.grid;
    if (c->neg.mode != OBGC_NEGATIVES_NONE) {
        // the state entering the first stage has been through update_state! (iteration 0); applying
        // the modifier again to a state it already produced changes nothing
        rc = launch_negatives(c->neg, sizeof(TS), cur, grid, st);
        if (rc == OBGC_OK && c->neg_passive.mode != OBGC_NEGATIVES_NONE)
            rc = launch_negatives(c->neg_passive, sizeof(TS), cur + c->NT, grid, st);
        if (rc != OBGC_OK) return rc;
    }
    // the sediment's coupled tendencies of the entering state
    rc = launch_multig<TS>(c, cur, 0.0, st);
    if (rc != OBGC_OK) return rc;
    for (int s = 0; s < nsteps; s++) {
        for (int stg = 0; stg < 3; stg++) {
            rc = enqueue_stage<TS, TC>(c, p, stg, cur, nxt, st, profile, ev);
            if (rc != OBGC_OK) return rc;
            for (int t = 0; t < NS; t++) { void* tmp = cur[t]; cur[t] = nxt[t]; nxt[t] = tmp; }
            // update_state! after the substep: the sediment tracks the new state and steps the stage
            rc = launch_multig<TS>(c, cur, (rk3_gamma(stg) + rk3_zeta(stg)) * dt, st);
            if (rc != OBGC_OK) return rc;
        }
        if (clock) {
            advance_time_kernel<<<1, 1, 0, st>>>(c->d_time, dt);
            OBGC_LAUNCHED("advance_time_kernel");
        }
    }
    if (nsteps % 2 == 1) {
        const obgc_grid& g = c->desc.grid;
        const int64_t N = (int64_t)g.Nx * g.Ny * g.Nz;
        for (int t = 0; t < NS; t++) {
            copy_interior_kernel<TS><<<(unsigned)((N + 255) / 256), 256, 0, st>>>((const TS*)cur[t], (TS*)c->user[t], g.Nx,
                                                                                g.Ny, g.Nz, g.stride_j, g.stride_k);
            OBGC_LAUNCHED("copy_interior_kernel");
        }
    }
    return OBGC_OK;
}

// One RK3 stage from caller arrays `in` into caller arrays `out` (the bound grid's layout).
template <typename TS, typename TC>
static int enqueue_one_stage(obgc_ctx* c, const FusedEntry* fe, double dt, int stage, const void* const* in,
                             void* const* out, cudaStream_t st) {
    StepPlan<TS, TC> p;
    int rc = plan_steps<TS, TC>(c, fe, dt, p);
    if (rc != OBGC_OK) return rc;
    rc = launch_thomas<TS, TC>(c, p, dt, st);
    if (rc != OBGC_OK) return rc;
    size_t ev = 0;
    return enqueue_stage<TS, TC>(c, p, stage, const_cast<void* const*>(in), out, st, false, ev);
}

static int dispatch_steps(obgc_ctx* c, double dt, int nsteps, cudaStream_t st, bool profile) {
    const FusedEntry* fe = c->V >= 0 ? find_fused(c->prec, c->V, c->NT) : nullptr;
    if (!fe) return fail(OBGC_ERR_UNSUPPORTED, "obgc_step: no fused kernel for this model variant / tracer set");
    if (c->prec == OBGC_PREC_F32) return enqueue_steps<float, float>(c, fe, dt, nsteps, st, profile);
    if (c->prec == OBGC_PREC_F64) return enqueue_steps<double, double>(c, fe, dt, nsteps, st, profile);
    return enqueue_steps<double, float>(c, fe, dt, nsteps, st, profile);
}

extern "C" int obgc_substep(obgc_ctx* c, double t, double dt, int32_t stage, const void* const* in, void* const* out,
                            void* stream) {
    if (!c || !c->bound) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_substep: context not bound");
    if (stage < 0 || stage > 2 || !(dt > 0) || !in || !out)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_substep: bad stage, dt or field arrays");
    if (c->mg_on) return fail(OBGC_ERR_UNSUPPORTED, "obgc_substep: the SimpleMultiG sediment steps with obgc_step only");
    const int NS = c->NT + c->NP;
    for (int q = 0; q < NS; q++)
        if (!in[q] || !out[q] || in[q] == out[q])
            return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_substep: every slot needs distinct input and output arrays");
    const FusedEntry* fe = c->V >= 0 ? find_fused(c->prec, c->V, c->NT) : nullptr;
    if (!fe) return fail(OBGC_ERR_UNSUPPORTED, "obgc_substep: no fused kernel for this model variant / tracer set");
    cudaStream_t st = (cudaStream_t)stream;
    OBGC_CUDA(cudaEventRecord(c->ev_begin, st));
    // the step's start time; the status word is cleared by the first stage and collects all three
    set_time_kernel<<<1, 1, 0, st>>>(c->d_time, t, stage == 0 ? c->d_status : nullptr);
    OBGC_LAUNCHED("set_time_kernel");
    int rc;
    if (c->prec == OBGC_PREC_F32) rc = enqueue_one_stage<float, float>(c, fe, dt, stage, in, out, st);
    else if (c->prec == OBGC_PREC_F64) rc = enqueue_one_stage<double, double>(c, fe, dt, stage, in, out, st);
    else rc = enqueue_one_stage<double, float>(c, fe, dt, stage, in, out, st);
    if (rc != OBGC_OK) return rc;
    OBGC_CUDA(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    OBGC_CUDA(cudaEventRecord(c->ev_end, st));
    return c->status_check ? obgc_step_status(c, nullptr) : OBGC_OK;
}

extern "C" int obgc_set_staging(obgc_ctx* c, int32_t mode) {
    if (!c || mode < 0 || mode > 1) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_staging: bad argument");
    c->staging = mode;
    return OBGC_OK;
}

extern "C" int obgc_get_staging(const obgc_ctx* c, int32_t* available, int32_t* last_used) {
    if (!c) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_get_staging: no context");
    if (available) *available = c->tma_ready ? 1 : 0;
    if (last_used) *last_used = c->last_used_tma ? 1 : 0;
    return OBGC_OK;
}

static int64_t launches_per_call(const obgc_ctx* c, int nsteps) {
    const bool clock = needs_clock(c);
    const int neg = c->neg.mode == OBGC_NEGATIVES_NONE ? 0 : c->neg_passive.mode != OBGC_NEGATIVES_NONE ? 2 : 1;
    int gases = 0;
    for (const auto& gc : c->gas) gases = gases || gc.on ? 1 : 0;   // one launch for all conditions
    const bool impl = c->vimplicit && c->kzf;
    const int per_stage = 1 + c->nchunk + gases + (impl ? 1 + neg : 0) + (c->mg_on ? 1 : 0) + (c->prefix_on ? 1 : 0) +
                          (c->last_used_tma && c->sinkpre_on ? 1 : 0);
    return (c->mg_on ? 1 : 0) + (int64_t)nsteps * (3 * per_stage + (clock ? 1 : 0)) + (c->last_used_tma && c->copied_first ? 1 : 0) +
           (nsteps % 2 && !c->last_used_tma ? c->NT + c->NP : 0) + 1 + neg + (impl ? 1 : 0);
}

extern "C" int obgc_step(obgc_ctx* c, double t, double dt, int32_t nsteps, void* stream) {
    if (!c || !c->bound) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_step: context not bound");
    if (nsteps < 0 || !(dt > 0)) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_step: bad dt / nsteps");
    cudaStream_t st = (cudaStream_t)stream;
    if (c->profile) {
        const size_t need = (size_t)6 * nsteps;
        while (c->prof_events.size() < need) {
            cudaEvent_t e;
            OBGC_CUDA(cudaEventCreate(&e));
            c->prof_events.push_back(e);
        }
    }
    OBGC_CUDA(cudaEventRecord(c->ev_begin, st));
    set_time_kernel<<<1, 1, 0, st>>>(c->d_time, t, c->d_status);
    OBGC_LAUNCHED("set_time_kernel");
    int rc = dispatch_steps(c, dt, nsteps, st, c->profile);
    if (rc != OBGC_OK) return rc;
    OBGC_CUDA(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    OBGC_CUDA(cudaEventRecord(c->ev_end, st));
    c->last_launches = launches_per_call(c, nsteps);
    if (c->profile) {
        OBGC_CUDA(cudaEventSynchronize(c->ev_end));
        float ms = 0;
        OBGC_CUDA(cudaEventElapsedTime(&ms, c->ev_begin, c->ev_end));
        c->last_total_ms = ms;
        double sub = 0;
        for (size_t q = 0; q + 1 < (size_t)6 * nsteps; q += 2) {
            float m = 0;
            OBGC_CUDA(cudaEventElapsedTime(&m, c->prof_events[q], c->prof_events[q + 1]));
            sub += m;
        }
        c->last_substep_ms = sub;
    }
    return c->status_check ? obgc_step_status(c, nullptr) : OBGC_OK;
}

extern "C" int obgc_step_graph(obgc_ctx* c, double t, double dt, int32_t nsteps, void* stream) {
    if (!c || !c->bound) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_step_graph: context not bound");
    if (nsteps < 1 || !(dt > 0)) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_step_graph: bad dt / nsteps");
    cudaStream_t st = (cudaStream_t)stream;
    if (!c->graph || c->graph_dt != dt || c->graph_nsteps != nsteps || c->graph_version != c->bind_version) {
        if (c->graph) { cudaGraphExecDestroy(c->graph); c->graph = nullptr; }
        cudaStream_t cap;
        OBGC_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
        cudaGraph_t graph;
        cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) { cudaStreamDestroy(cap); return cuda_fail(e, "cudaStreamBeginCapture"); }
        int rc = dispatch_steps(c, dt, nsteps, cap, false);
        e = cudaStreamEndCapture(cap, &graph);
        cudaStreamDestroy(cap);
        if (rc != OBGC_OK) { if (e == cudaSuccess) cudaGraphDestroy(graph); return rc; }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture");
        e = cudaGraphInstantiate(&c->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
        c->graph_dt = dt;
        c->graph_nsteps = nsteps;
        c->graph_version = c->bind_version;
    }
    OBGC_CUDA(cudaEventRecord(c->ev_begin, st));
    set_time_kernel<<<1, 1, 0, st>>>(c->d_time, t, c->d_status);
    OBGC_LAUNCHED("set_time_kernel");
    OBGC_CUDA(cudaGraphLaunch(c->graph, st));
    count_launches(launches_per_call(c, nsteps) - 1);
    OBGC_CUDA(cudaMemcpyAsync(c->h_status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    OBGC_CUDA(cudaEventRecord(c->ev_end, st));
    c->last_launches = launches_per_call(c, nsteps);
    return OBGC_OK;
}

extern "C" int obgc_step_status(obgc_ctx* c, int32_t* flags) {
    if (!c || !c->h_status) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_step_status: no context");
    OBGC_CUDA(cudaEventSynchronize(c->ev_end));
    const int f = *c->h_status;
    if (flags) *flags = f;
    if (f & OBGC_FLAG_NAN) return fail(OBGC_ERR_NAN, "obgc_step: a substep wrote a NaN or an infinity into the state");
    if (f & OBGC_FLAG_NOT_CONVERGED)
        return fail(OBGC_ERR_NOT_CONVERGED, "obgc_step: a surface pCO2 solve of the gas exchange did not converge");
    if (f & OBGC_FLAG_TIMEOUT)
        return fail(OBGC_ERR_TIMEOUT, "obgc_step: a block stopped waiting for its tile copies (tensor-memory accelerator)");
    return OBGC_OK;
}

extern "C" int obgc_set_status_check(obgc_ctx* c, int32_t on) {
    if (!c) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_set_status_check: no context");
    c->status_check = on != 0;
    return OBGC_OK;
}

// Device copies of everything an obgc_step call carries into the next one (the bound tracers, the
// sediment storages and the gas exchange's warm-start [H+]), taken before the autotuner's trial
// steps and written back after them; freed on every return path.
struct StepSnapshot {
    struct Piece {
        void* live;
        void* copy;
        size_t bytes;
    };
    std::vector<Piece> pieces;
    ~StepSnapshot() {
        for (auto& p : pieces) cudaFree(p.copy);
    }
    int add(void* live, size_t bytes) {
        if (!live || !bytes) return OBGC_OK;
        Piece p{live, nullptr, bytes};
        OBGC_CUDA(cudaMalloc(&p.copy, bytes));
        pieces.push_back(p);
        return OBGC_OK;
    }
    int save(cudaStream_t st) {
        for (auto& p : pieces) OBGC_CUDA(cudaMemcpyAsync(p.copy, p.live, p.bytes, cudaMemcpyDeviceToDevice, st));
        return OBGC_OK;
    }
    int restore(cudaStream_t st) {
        for (auto& p : pieces) OBGC_CUDA(cudaMemcpyAsync(p.live, p.copy, p.bytes, cudaMemcpyDeviceToDevice, st));
        return OBGC_OK;
    }
};

extern "C" int obgc_autotune_step(obgc_ctx* c, double t, double dt, int32_t steps, int32_t* levels_per_item,
                                  int32_t* staging, double* ms_per_step, void* stream) {
    if (!c || !c->bound) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_autotune_step: context not bound");
    if (steps < 1 || !(dt > 0)) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_autotune_step: bad dt / steps");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const obgc_grid& g = c->desc.grid;
    const int64_t cols = (int64_t)g.Nx * g.Ny;
    // the span of a bound field the kernels touch: its last cell is (Nx-1, Ny-1, Nz-1)
    const int64_t span = (int64_t)g.stride_k * (g.Nz - 1) + (int64_t)g.stride_j * (g.Ny - 1) + g.Nx;
    StepSnapshot snap;
    for (int t = 0; t < c->NT + c->NP; t++) {
        const int rc = snap.add(c->user[t], c->ts * span);
        if (rc != OBGC_OK) return rc;
    }
    int rc = snap.add(c->sed_storage, c->ts * cols);
    if (rc == OBGC_OK) rc = snap.add(c->mg_state, sizeof(double) * 4 * cols);
    for (const auto& gc : c->gas)
        if (rc == OBGC_OK && gc.on) rc = snap.add(gc.H, sizeof(double) * cols);
    if (rc == OBGC_OK) rc = snap.save(st);
    if (rc != OBGC_OK) return rc;

    const int TZ0 = c->TZ, staging0 = c->staging;
    const bool profile0 = c->profile, check0 = c->status_check;
    c->profile = false;
    c->status_check = true;
    // the candidates: levels per work item, each with both tile stagings where the tensor copies exist
    std::vector<int> tzs;
    for (int tz : {2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 16, 24, 32}) {
        const int v = std::min(tz, g.Nz);
        if (std::find(tzs.begin(), tzs.end(), v) == tzs.end()) tzs.push_back(v);
    }
    double best = 1e300;
    int best_tz = TZ0, best_staging = staging0;
    for (int tz : tzs) {
        for (int sg = c->tma_ready ? 1 : 0; sg >= 0 && rc == OBGC_OK; sg--) {
            c->TZ = tz;
            c->staging = sg;
            // one warm-up step, then the timed steps; each candidate from the saved state
            rc = obgc_step(c, t, dt, 1, stream);
            if (rc == OBGC_OK) rc = snap.restore(st);
            if (rc != OBGC_OK) break;
            rc = obgc_step(c, t, dt, steps, stream);
            if (rc != OBGC_OK) break;
            float ms = 0;
            const cudaError_t e = cudaEventElapsedTime(&ms, c->ev_begin, c->ev_end);
            if (e != cudaSuccess) { rc = cuda_fail(e, "cudaEventElapsedTime"); break; }
            if (ms < best) { best = ms; best_tz = tz; best_staging = sg; }
            rc = snap.restore(st);
        }
        if (rc != OBGC_OK) break;
    }
    const int rc_restore = snap.restore(st);
    const cudaError_t e_sync = cudaStreamSynchronize(st);
    c->profile = profile0;
    c->status_check = check0;
    c->graph_version = ~0ull;
    if (rc != OBGC_OK) {
        c->TZ = TZ0;
        c->staging = staging0;
        return rc;
    }
    if (rc_restore != OBGC_OK) return rc_restore;
    if (e_sync != cudaSuccess) return cuda_fail(e_sync, "cudaStreamSynchronize");
    c->TZ = best_tz;
    c->staging = best_staging;
    if (levels_per_item) *levels_per_item = best_tz;
    if (staging) *staging = best_staging;
    if (ms_per_step) *ms_per_step = best / steps;
    return OBGC_OK;
}

extern "C" int obgc_last_step_timing(const obgc_ctx* c, double* total_ms, double* substep_ms, int64_t* launches) {
    if (!c) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_last_step_timing: null context");
    if (!c->profile) {
        float ms = 0;
        OBGC_CUDA(cudaEventSynchronize(c->ev_end));
        OBGC_CUDA(cudaEventElapsedTime(&ms, c->ev_begin, c->ev_end));
        if (total_ms) *total_ms = ms;
        if (substep_ms) *substep_ms = 0;
    } else {
        if (total_ms) *total_ms = c->last_total_ms;
        if (substep_ms) *substep_ms = c->last_substep_ms;
    }
    if (launches) *launches = c->last_launches;
    return OBGC_OK;
}

template <typename TS>
static int launch_budget(obgc_ctx* c, const int* names, const double* scale, int n, double* total, cudaStream_t st) {
    BudgetArgs<TS> b;
    std::memset(&b, 0, sizeof(b));
    b.n = n;
    for (int q = 0; q < n; q++) {
        b.f[q] = (const TS*)c->fields.tracers[names[q]];
        if (!b.f[q]) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_tracer_budget: conserved tracer not bound");
        b.scale[q] = scale[q];
    }
    const obgc_grid& g = c->desc.grid;
    budget_partial_kernel<TS><<<c->n_partial, BUDGET_THREADS, 0, st>>>(b, g.Nx, g.Ny, g.Nz, g.stride_j, g.stride_k, c->partial);
    OBGC_LAUNCHED("budget_partial_kernel");
    budget_final_kernel<<<1, BUDGET_THREADS, 0, st>>>(c->partial, c->n_partial, c->d_budget);
    OBGC_LAUNCHED("budget_final_kernel");
    OBGC_CUDA(cudaMemcpyAsync(total, c->d_budget, sizeof(double), cudaMemcpyDeviceToHost, st));
    OBGC_CUDA(cudaStreamSynchronize(st));
    return OBGC_OK;
}

extern "C" int obgc_tracer_budget(obgc_ctx* c, int32_t group, double* total, void* stream) {
    if (!c || !c->bound || !total || (group != 0 && group != 1))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_tracer_budget: bad argument");
    int names[16];
    double scale[16];
    const int n = conserved_group(c->desc.npd, group, names, scale);
    if (n < 0) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_tracer_budget: model has no carbonate system");
    if (n > BUDGET_MAX_TRACERS) return fail(OBGC_ERR_UNSUPPORTED, "obgc_tracer_budget: too many tracers");
    cudaStream_t st = (cudaStream_t)stream;
    if (c->ts == 4) return launch_budget<float>(c, names, scale, n, total, st);
    return launch_budget<double>(c, names, scale, n, total, st);
}
