// light.cu — TwoBand / MultiBand PAR and euphotic depth (src/Light).
//
// Layout: i-fastest fields, so one thread per (i, j) column marching k from the surface down
// gives fully coalesced 128-byte row accesses per warp at every level (the reference launches the
// same :xy work with one thread per column, 2band.jl:151).  MultiBand computes every band in one
// pass over the chlorophyll field instead of one launch per band (multi_band.jl:170-180).
#include <cmath>
#include <vector>
#include "light_device.cuh"

namespace obgc {

template <typename T>
__device__ __forceinline__ T surface_value(int kind, T value, const T* field, int64_t col) {
    return kind == OBGC_SURFACE_PAR_FIELD ? field[col] : value;
}

template <typename T>
__global__ void __launch_bounds__(128) twoband_kernel(TwoBandT<T> L, int surf_kind, T surf_value,
                                                      const T* __restrict__ surf_field, int Nx, int Ny,
                                                      int Nz, int64_t sj, int64_t sk, T Lz,
                                                      const T* __restrict__ P, T* __restrict__ PAR) {
    const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= (int64_t)Nx * Ny) return;
    const int i = (int)(col % Nx), j = (int)(col / Nx);
    const T dz = Lz / T(Nz);
    const T PAR0 = surface_value(surf_kind, surf_value, surf_field, col);
    const int64_t base = i + (int64_t)j * sj;
    T Sr = T(0), Sb = T(0);
    for (int k = Nz - 1; k >= 0; --k) {
        const int64_t idx = base + (int64_t)k * sk;
        T fr, fb;
        twoband_terms(L, P[idx], fr, fb);
        const T z = -Lz + (T(k) + T(0.5)) * dz;
        PAR[idx] = twoband_par(L, PAR0, z, dz, Sr, Sb, fr, fb);
        Sr += fr;
        Sb += fb;
    }
}

constexpr int MAX_BANDS = 8;
// Fields in the storage type TS, arithmetic in T (FP32 for a model whose state is FP64 and whose
// light runs in FP32).
template <typename T, typename TS = T>
struct BandsT {
    int n;
    T kw[MAX_BANDS], e[MAX_BANDS], chi[MAX_BANDS], div[MAX_BANDS];
    TS* out[MAX_BANDS];
};

// One warp per column: each lane takes one level of a 32-level chunk (top first), the attenuation
// factor of its level, and a multiplicative shuffle scan down the chunk continues the product carried
// from the chunk above (multi_band.jl:147-185: PAR at the top cell PAR0 div exp(z att), below it
// the cell above times exp((z - z_above) att)).
template <typename T, typename TS = T>
__global__ void __launch_bounds__(128) multiband_kernel(BandsT<T, TS> B, int surf_kind, T surf_value,
                                                        const TS* __restrict__ surf_field, int Nx, int Ny,
                                                        int Nz, int64_t sj, int64_t sk, T Lz,
                                                        const TS* __restrict__ Chl, TS* __restrict__ total) {
    const int lane = threadIdx.x & 31;
    const int64_t col = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (col >= (int64_t)Nx * Ny) return;   // warp-uniform
    const int i = (int)(col % Nx), j = (int)(col / Nx);
    const T dz = Lz / T(Nz);
    const T PAR0 = surf_kind == OBGC_SURFACE_PAR_FIELD ? T(surf_field[col]) : surf_value;
    const int64_t base = i + (int64_t)j * sj;
    T carry[MAX_BANDS];
#pragma unroll
    for (int b = 0; b < MAX_BANDS; b++) carry[b] = T(1);
    for (int k0 = 0; k0 < Nz; k0 += 32) {
        const int k = Nz - 1 - (k0 + lane);
        const bool valid = k >= 0;
        const int64_t idx = base + (int64_t)(valid ? k : 0) * sk;
        const T chl = valid ? T(Chl[idx]) : T(0);
        const T z = -Lz + (T(k) + T(0.5)) * dz;
        T sum = T(0);
#pragma unroll
        for (int b = 0; b < MAX_BANDS; b++) {
            if (b < B.n) {
                const T att = B.kw[b] + B.chi[b] * t_pow(chl, B.e[b]);
                T f = T(1);
                if (valid) f = (k == Nz - 1) ? PAR0 * B.div[b] * t_exp(z * att) : t_exp(-dz * att);
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const T fp = __shfl_up_sync(0xffffffffu, f, o);
                    if (lane >= o) f *= fp;
                }
                const T v = carry[b] * f;
                if (valid) B.out[b][idx] = TS(v);
                sum += v;
                carry[b] = __shfl_sync(0xffffffffu, v, 31);
            }
        }
        if (total && valid) total[idx] = TS(sum);
    }
}

template <typename T>
__global__ void __launch_bounds__(128) euphotic_kernel(int surf_kind, T surf_value, const T* __restrict__ surf_field,
                                                       int Nx, int Ny, int Nz, int64_t sj, int64_t sk, T Lz,
                                                       T cutoff, const T* __restrict__ PAR, T* __restrict__ zeu) {
    const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= (int64_t)Nx * Ny) return;
    const int i = (int)(col % Nx), j = (int)(col / Nx);
    const T dz = Lz / T(Nz);
    const T surface = surface_value(surf_kind, surf_value, surf_field, col);
    const int64_t base = i + (int64_t)j * sj;
    bool found = false;
    T z_eu = T(0);
    // compute_euphotic_depth.jl:13-25: the last assignment in the downward scan is the first
    // crossing from the top, so stop at the first crossing.
    for (int k = Nz - 2; k >= 0 && !found; --k) {
        const T Pk = PAR[base + (int64_t)k * sk];
        if (Pk <= surface * cutoff) {
            const T Pk1 = PAR[base + (int64_t)(k + 1) * sk];
            const T zk = -Lz + (T(k) + T(0.5)) * dz, zk1 = zk + dz;
            z_eu = zk + (log(surface * cutoff) - log(Pk)) * (zk - zk1) / (log(Pk) - log(Pk1));
            found = true;
        }
    }
    if (!found || !isfinite(z_eu)) z_eu = -Lz - T(0.5) * dz;
    zeu[col] = z_eu;
}

template <typename T>
static int launch_twoband(const obgc_twoband_params* lp, const obgc_surface* s, const obgc_grid* g,
                          const void* P, void* PAR, double t, cudaStream_t st) {
    const int64_t ncol = (int64_t)g->Nx * g->Ny;
    const int threads = 128;
    const int blocks = (int)((ncol + threads - 1) / threads);
    const double v = s->kind == OBGC_SURFACE_PAR_DEFAULT ? default_surface_par(t) : s->value;
    twoband_kernel<T><<<blocks, threads, 0, st>>>(make_twoband<T>(*lp), s->kind, T(v), (const T*)s->field,
                                                  g->Nx, g->Ny, g->Nz, g->stride_j, g->stride_k, T(g->Lz),
                                                  (const T*)P, (T*)PAR);
    OBGC_LAUNCHED("twoband_kernel");
    return OBGC_OK;
}

template <typename T, typename TS = T>
static int launch_multiband(int nb, const double* kw, const double* e, const double* chi, const double* dv,
                            const obgc_surface* s, const obgc_grid* g, const void* Chl,
                            void* const* bands, void* total, double t, cudaStream_t st) {
    BandsT<T, TS> B;
    B.n = nb;
    for (int b = 0; b < nb; b++) {
        B.kw[b] = T(kw[b]); B.e[b] = T(e[b]); B.chi[b] = T(chi[b]); B.div[b] = T(dv[b]);
        B.out[b] = (TS*)bands[b];
    }
    const int64_t ncol = (int64_t)g->Nx * g->Ny;
    const int blocks = (int)((ncol * 32 + 127) / 128);   // one warp per column
    const double v = s->kind == OBGC_SURFACE_PAR_DEFAULT ? default_surface_par(t) : s->value;
    multiband_kernel<T, TS><<<blocks, 128, 0, st>>>(B, s->kind, T(v), (const TS*)s->field, g->Nx, g->Ny, g->Nz,
                                                    g->stride_j, g->stride_k, T(g->Lz), (const TS*)Chl, (TS*)total);
    OBGC_LAUNCHED("multiband_kernel");
    return OBGC_OK;
}

template <typename T>
static int launch_euphotic(const obgc_surface* s, const obgc_grid* g, const void* PAR, void* zeu,
                           double cutoff, double t, cudaStream_t st) {
    const int64_t ncol = (int64_t)g->Nx * g->Ny;
    const int blocks = (int)((ncol + 127) / 128);
    const double v = s->kind == OBGC_SURFACE_PAR_DEFAULT ? default_surface_par(t) : s->value;
    euphotic_kernel<T><<<blocks, 128, 0, st>>>(s->kind, T(v), (const T*)s->field, g->Nx, g->Ny, g->Nz,
                                               g->stride_j, g->stride_k, T(g->Lz), T(cutoff), (const T*)PAR, (T*)zeu);
    OBGC_LAUNCHED("euphotic_kernel");
    return OBGC_OK;
}

static bool valid_surface(const obgc_surface* s) {
    if (!s) return false;
    if (s->kind == OBGC_SURFACE_PAR_FIELD) return s->field != nullptr;
    return s->kind == OBGC_SURFACE_PAR_DEFAULT || s->kind == OBGC_SURFACE_PAR_CONSTANT;
}

}  // namespace obgc

using namespace obgc;

extern "C" int obgc_twoband_par(const obgc_twoband_params* lp, const obgc_surface* surface,
                                const obgc_grid* grid, int32_t dtype, const void* P, void* PAR,
                                double t, void* stream) {
    if (!lp || !valid_surface(surface) || !valid_grid(grid) || !P || !PAR)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_twoband_par: bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == OBGC_F32) return launch_twoband<float>(lp, surface, grid, P, PAR, t, st);
    if (dtype == OBGC_F64) return launch_twoband<double>(lp, surface, grid, P, PAR, t, st);
    return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_twoband_par: bad dtype");
}

extern "C" int obgc_multiband_par(int32_t nbands, const double* kw, const double* e, const double* chi,
                                  const double* division, const obgc_surface* surface,
                                  const obgc_grid* grid, int32_t dtype, const void* Chl,
                                  void* const* band_fields, void* PAR_total, double t, void* stream) {
    if (nbands < 1 || nbands > MAX_BANDS || !kw || !e || !chi || !division || !band_fields || !Chl ||
        !valid_surface(surface) || !valid_grid(grid))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_multiband_par: bad argument");
    double sum = 0;
    for (int b = 0; b < nbands; b++) {
        if (!band_fields[b]) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_multiband_par: null band field");
        sum += division[b];
    }
    // multi_band.jl:106
    if (sum != 1.0) return fail(OBGC_ERR_INVALID_ARGUMENT, "surface_PAR_division does not sum to 1");
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == OBGC_F32) return launch_multiband<float>(nbands, kw, e, chi, division, surface, grid, Chl, band_fields, PAR_total, t, st);
    if (dtype == OBGC_F64) return launch_multiband<double>(nbands, kw, e, chi, division, surface, grid, Chl, band_fields, PAR_total, t, st);
    return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_multiband_par: bad dtype");
}

extern "C" int obgc_multiband_coefficients(int32_t nbands, const double* edges, int32_t nbase,
                                           const double* lambda, const double* bkw, const double* be,
                                           const double* bchi, double* kw, double* e, double* chi) {
    if (nbands < 1 || nbase < 2 || !edges || !lambda || !bkw || !be || !bchi || !kw || !e || !chi)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_multiband_coefficients: bad argument");
    for (int b = 0; b < nbands; b++) {
        // findlast(base_bands .<= edge) (multi_band.jl:98-99)
        int i1 = -1, i2 = -1;
        for (int n = 0; n < nbase; n++) {
            if (lambda[n] <= edges[2 * b]) i1 = n;
            if (lambda[n] <= edges[2 * b + 1]) i2 = n;
        }
        if (i1 < 0 || i2 <= i1) return fail(OBGC_ERR_INVALID_ARGUMENT, "band outside the base wavelengths");
        // numerical_mean (multi_band.jl:136-140): trapezoidal mean over [lambda_i1, lambda_i2]
        const double* src[3] = {bkw, be, bchi};
        double* dst[3] = {kw, e, chi};
        for (int q = 0; q < 3; q++) {
            double s = 0.0;
            for (int n = i1 + 1; n <= i2; n++) s += (src[q][n] + src[q][n - 1]) * (lambda[n] - lambda[n - 1]) / 2;
            dst[q][b] = s / (lambda[i2] - lambda[i1]);
        }
    }
    return OBGC_OK;
}

extern "C" int obgc_euphotic_depth(const obgc_surface* surface, const obgc_grid* grid, int32_t dtype,
                                   const void* PAR, void* zeu, double cutoff, double t, void* stream) {
    if (!valid_surface(surface) || !valid_grid(grid) || !PAR || !zeu)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_euphotic_depth: bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == OBGC_F32) return launch_euphotic<float>(surface, grid, PAR, zeu, cutoff, t, st);
    if (dtype == OBGC_F64) return launch_euphotic<double>(surface, grid, PAR, zeu, cutoff, t, st);
    return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_euphotic_depth: bad dtype");
}

namespace obgc {
// FP64 fields, FP32 arithmetic: the MultiBand light of a model whose state is FP64 and whose light
// runs in FP32 (OBGC_PREC_MIXED).  Arguments as obgc_multiband_par, already validated.
int multiband_par_mixed(int nb, const double* kw, const double* e, const double* chi, const double* dv,
                        const obgc_surface* s, const obgc_grid* g, const void* Chl, void* const* bands, void* total,
                        double t, cudaStream_t st) {
    return launch_multiband<float, double>(nb, kw, e, chi, dv, s, g, Chl, bands, total, t, st);
}
}  // namespace obgc
