// gas.cu — air-sea gas exchange fluxes of every column (GasExchange boundary conditions).
#include <cstring>
#include "gas_device.cuh"

namespace obgc {

// One thread per column: the surface cell (k = Nz - 1) of T, S and DIC/Alk or O2.
template <typename T>
__global__ void __launch_bounds__(128) gas_exchange_kernel(obgc_gas_exchange g, int Nx, int Ny, int Nz, int64_t sj,
                                                           int64_t sk, const T* __restrict__ Tc, const T* __restrict__ S,
                                                           const T* __restrict__ DIC, const T* __restrict__ Alk,
                                                           const T* __restrict__ O2, const T* __restrict__ wind,
                                                           const T* __restrict__ air, double* __restrict__ flux,
                                                           double* __restrict__ H) {
    const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= (int64_t)Nx * Ny) return;
    const int i = (int)(col % Nx), j = (int)(col / Nx);
    const int64_t o = i + (int64_t)j * sj + (int64_t)(Nz - 1) * sk;
    const double u10 = wind ? (double)wind[col] : g.wind_speed;
    const double ca = air ? (double)air[col] : g.air_concentration;
    const bool co2 = g.gas == OBGC_GAS_CO2;
    flux[col] = gas_flux_cell(g, (double)Tc[o], (double)S[o], co2 ? (double)DIC[o] : 0.0, co2 ? (double)Alk[o] : 0.0,
                              co2 ? 0.0 : (double)O2[o], u10, ca, H ? H + col : nullptr);
}

template <typename T>
__global__ void __launch_bounds__(128) gas_exchange_multi_kernel(const __grid_constant__ GasMulti m, int Nx, int Ny, int Nz,
                                                                 int64_t sj, int64_t sk, const T* __restrict__ Tc,
                                                                 const T* __restrict__ S) {
    const int64_t col = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (col >= (int64_t)Nx * Ny) return;
    const int i = (int)(col % Nx), j = (int)(col / Nx);
    const int64_t o = i + (int64_t)j * sj + (int64_t)(Nz - 1) * sk;
    const double Tv = (double)Tc[o], Sv = (double)S[o];
    Co2Column shared;
    bool prepared = false;
    for (int q = 0; q < m.n; q++) {
        const obgc_gas_exchange& g = m.g[q];
        const double u10 = g.wind_field ? (double)static_cast<const T*>(g.wind_field)[col] : g.wind_speed;
        const double ca = g.air_field ? (double)static_cast<const T*>(g.air_field)[col] : g.air_concentration;
        if (g.gas != OBGC_GAS_CO2) {
            m.flux[q][col] = gas_flux_cell(g, Tv, Sv, 0.0, 0.0, (double)static_cast<const T*>(m.O2[q])[o], u10, ca);
            continue;
        }
        double* Hq = m.H[q] + col;
        if (!(Hq[0] > 0.0)) Hq[0] = exp(-2.302585092994046 * g.carbon.initial_pH_guess);
        const double DIC = (double)static_cast<const T*>(m.DIC[q])[o], Alk = (double)static_cast<const T*>(m.Alk[q])[o];
        if (m.share[q]) {
            if (!prepared) {
                co2_column_prepare(g, Tv, Sv, u10, shared);
                prepared = true;
            }
            shared.k_sol = co2_k_sol(g, Tv, shared.sol, u10);
            bool ok = true;
            m.flux[q][col] = co2_column_flux(g, shared, DIC, Alk, ca, Hq[0], &ok);
            if (!ok && m.status) atomicOr(m.status, OBGC_FLAG_NOT_CONVERGED);
        } else {
            Co2Column own;
            co2_column_prepare(g, Tv, Sv, u10, own);
            bool ok = true;
            m.flux[q][col] = co2_column_flux(g, own, DIC, Alk, ca, Hq[0], &ok);
            if (!ok && m.status) atomicOr(m.status, OBGC_FLAG_NOT_CONVERGED);
        }
    }
}

template <typename T>
int launch_gas_exchange_multi(const GasMulti& m, const obgc_grid* grid, const void* Tc, const void* S, cudaStream_t st) {
    const int64_t cols = (int64_t)grid->Nx * grid->Ny;
    gas_exchange_multi_kernel<T><<<(unsigned)((cols + 127) / 128), 128, 0, st>>>(m, grid->Nx, grid->Ny, grid->Nz,
                                                                              grid->stride_j, grid->stride_k,
                                                                              (const T*)Tc, (const T*)S);
    OBGC_LAUNCHED("gas_exchange_multi_kernel");
    return OBGC_OK;
}
template int launch_gas_exchange_multi<float>(const GasMulti&, const obgc_grid*, const void*, const void*, cudaStream_t);
template int launch_gas_exchange_multi<double>(const GasMulti&, const obgc_grid*, const void*, const void*, cudaStream_t);

template <typename T>
int launch_gas_exchange(const obgc_gas_exchange* g, const obgc_grid* grid, const void* Tc, const void* S,
                        const void* DIC, const void* Alk, const void* O2, double* flux, cudaStream_t st, double* H) {
    const int64_t cols = (int64_t)grid->Nx * grid->Ny;
    gas_exchange_kernel<T><<<(unsigned)((cols + 127) / 128), 128, 0, st>>>(
        *g, grid->Nx, grid->Ny, grid->Nz, grid->stride_j, grid->stride_k, (const T*)Tc, (const T*)S, (const T*)DIC,
        (const T*)Alk, (const T*)O2, (const T*)g->wind_field, (const T*)g->air_field, flux, H);
    OBGC_LAUNCHED("gas_exchange_kernel");
    return OBGC_OK;
}
template int launch_gas_exchange<float>(const obgc_gas_exchange*, const obgc_grid*, const void*, const void*,
                                        const void*, const void*, const void*, double*, cudaStream_t, double*);
template int launch_gas_exchange<double>(const obgc_gas_exchange*, const obgc_grid*, const void*, const void*,
                                         const void*, const void*, const void*, double*, cudaStream_t, double*);

bool valid_gas(const obgc_gas_exchange* g) {
    return g && (g->gas == OBGC_GAS_CO2 || g->gas == OBGC_GAS_O2);
}

}  // namespace obgc

using namespace obgc;

extern "C" int obgc_gas_exchange_defaults(int32_t gas, obgc_gas_exchange* g) {
    if (!g || (gas != OBGC_GAS_CO2 && gas != OBGC_GAS_O2)) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_gas_exchange_defaults: bad argument");
    std::memset(g, 0, sizeof(*g));
    g->gas = gas;
    g->k660[2] = 0.266 / 3600.0 / 100;   // Ho06 (gas_transfer_velocity.jl:53-59)
    g->wind_speed = 2.0;
    obgc_carbon_default_options(&g->carbon);
    g->carbon.output = OBGC_OUT_PCO2;
    if (gas == OBGC_GAS_CO2) {
        // CarbonDioxidePolynomialSchmidtNumber (schmidt_number.jl:6-7); 413 ppmv (GasExchange.jl:98)
        const double s[5] = {2116.8, -136.25, 4.7353, -0.092307, 0.0007555};
        std::memcpy(g->schmidt, s, sizeof(s));
        g->air_concentration = 413.0;
    } else {
        // OxygenPolynomialSchmidtNumber (schmidt_number.jl:14-15); OxygenSolubility
        // (gas_solubility.jl:52-53); 9352.7 mmol O2 / m3 (GasExchange.jl:141)
        const double s[5] = {1920.4, -135.6, 5.2122, -0.10939, 0.00093777};
        const double a[6] = {-58.3877, 85.8079, 23.8439, -0.034892, 0.015578, -0.0019387};
        std::memcpy(g->schmidt, s, sizeof(s));
        std::memcpy(g->o2_solubility, a, sizeof(a));
        g->air_concentration = 9352.7;
    }
    return OBGC_OK;
}

extern "C" int obgc_gas_exchange_flux(const obgc_gas_exchange* g, const obgc_grid* grid, int32_t dtype, const void* T,
                                      const void* S, const void* DIC, const void* Alk, const void* O2, double* flux,
                                      void* stream) {
    if (!valid_gas(g) || !valid_grid(grid) || !T || !S || !flux || (dtype != OBGC_F32 && dtype != OBGC_F64) ||
        (g->gas == OBGC_GAS_CO2 && (!DIC || !Alk)) || (g->gas == OBGC_GAS_O2 && !O2))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_gas_exchange_flux: bad argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return dtype == OBGC_F32 ? launch_gas_exchange<float>(g, grid, T, S, DIC, Alk, O2, flux, st, nullptr)
                             : launch_gas_exchange<double>(g, grid, T, S, DIC, Alk, O2, flux, st, nullptr);
}

extern "C" int obgc_gas_exchange_point(const obgc_gas_exchange* g, double T, double S, double DIC, double Alk, double O2,
                                       double u10, double air, double* flux) {
    if (!valid_gas(g) || !flux) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_gas_exchange_point: bad argument");
    *flux = gas_flux_cell(*g, T, S, DIC, Alk, O2, u10, air);
    return OBGC_OK;
}
