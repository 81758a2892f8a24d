// gas_device.cuh — air-sea gas exchange of one column's surface cell (host and device), FP64.
//
// GasExchange functor (src/Models/GasExchange/gas_exchange.jl:26-39): flux = k (C_water - C_air),
// positive out of the ocean, with k = k660(u10) / sqrt(Sc(T) / 660) * solubility(T, S)
// (gas_transfer_velocity.jl:30-31).
//   CO2: C_water = pCO2 of the surface DIC, Alk, T, S with silicate = phosphate = 0
//        (carbon_dioxide_concentration.jl:48-60), solubility = K0(T + 273.15, S) rho(T, S) / 1000
//        with the carbon chemistry's density function at zero pressure (gas_solubility.jl:58-65,
//        GasExchange.jl:110).
//   O2:  C_water = O2, C_air = air * beta / Tk of Wanninkhof92Solubility evaluated as the reference
//        writes it (gas_solubility.jl:40-50: B2 serves both salinity coefficients), solubility 1.
#pragma once
#include "carbon_device.cuh"

namespace obgc {

// H: when non-null, the Newton solve of the CO2 condition starts from *H if positive (the
// column's [H+] of the previous evaluation) and leaves the solved [H+] there; otherwise it starts
// from 10^-initial_pH_guess.
__host__ __device__ inline double gas_flux_cell(const obgc_gas_exchange& g, double T, double S, double DIC,
                                                double Alk, double O2, double u10, double air, double* H = nullptr) {
    const double k660 = g.k660[0] + u10 * (g.k660[1] + u10 * (g.k660[2] + u10 * g.k660[3]));
    const double Sc = g.schmidt[0] + T * (g.schmidt[1] + T * (g.schmidt[2] + T * (g.schmidt[3] + T * g.schmidt[4])));
    const double kS = k660 / sqrt(Sc / 660.0);
    if (g.gas == OBGC_GAS_CO2) {
        const double Tk = T + 273.15;
        const double solubility = weiss_k0(Tk, S, log(Tk), 1.0 / Tk) * seawater_density(g.carbon, T, S, 0.0) / 1000.0;
        obgc_carbon_options o = g.carbon;
        o.output = OBGC_OUT_PCO2;
        o.ph_given = 0;
        o.has_pressure = 0;
        const double H0 = H && *H > 0.0 ? *H : exp(-2.302585092994046 * o.initial_pH_guess);
        const double pCO2 = carbon_cell(o, DIC, Alk, T, S, 0.0, 0.0, 0.0, 0.0, H0, H, nullptr, nullptr);
        return kS * solubility * (pCO2 - air);
    }
    const double Tk = T + 273.15, Tk_100 = Tk / 100.0;
    const double* A = g.o2_solubility;
    const double beta = exp(A[0] + A[1] / Tk_100 + A[2] * log(Tk_100) + S * (A[3] + A[4] * Tk_100 + A[4] * (Tk_100 * Tk_100)));
    return kS * (O2 - air * (beta / Tk));
}

// The CO2 condition of one column whose surface T and S stay fixed (the column engine): the
// T/S-dependent parts of gas_flux_cell evaluated once (equilibrium constants, the residual's
// H-independent terms, the density conversion, k x solubility), then per RK3 stage only the
// unit conversion of DIC and Alk, the Newton solve started from the column's previous [H+], and
// pCO2.  The same arithmetic as gas_flux_cell but for the starting point of the solve.
struct Co2Column {
    CarbConsts c;
    double conv;       // 1e-3 / rho (mmol/m3 -> mol/kg)
    double k_sol;      // transfer velocity x solubility
    double Tk;
    double sol;        // solubility K0 rho(T, S, 0) / 1000
};

// Transfer velocity x solubility of condition g at wind u10 over water at T (degC), from the
// solubility the column's constants hold: the same product as gas_flux_cell forms.
__host__ __device__ inline double co2_k_sol(const obgc_gas_exchange& g, double T, double sol, double u10) {
    const double k660 = g.k660[0] + u10 * (g.k660[1] + u10 * (g.k660[2] + u10 * g.k660[3]));
    const double Sc = g.schmidt[0] + T * (g.schmidt[1] + T * (g.schmidt[2] + T * (g.schmidt[3] + T * g.schmidt[4])));
    return k660 / sqrt(Sc / 660.0) * sol;
}

__host__ __device__ inline void co2_column_prepare(const obgc_gas_exchange& g, double T, double S, double u10, Co2Column& col) {
    const double Tk = T + 273.15;
    col.Tk = Tk;
    col.sol = weiss_k0(Tk, S, log(Tk), 1.0 / Tk) * seawater_density(g.carbon, T, S, 0.0) / 1000.0;
    col.k_sol = co2_k_sol(g, T, col.sol, u10);
    col.conv = 1e-3 / seawater_density(g.carbon, T, S, 1.0);   // the pCO2 functor's density at 1 bar
    CarbConsts& c = col.c;
    c.boron = 0.000232 / 10.811 * S / 1.80655;
    c.sulfate = 0.14 / 96.06 * S / 1.80655;
    c.fluoride = 0.000067 / 18.9984 * S / 1.80655;
    c.DIC = c.Alk = c.phosphate = c.silicate = 0.0;
    equilibrium_constants(Tk, S, false, 0.0, true, c);
    prepare_residual(c);
}

// Flux (positive out of the ocean) from the surface DIC and Alk; H: the column's [H+], updated.
__host__ __device__ inline double co2_column_flux(const obgc_gas_exchange& g, const Co2Column& col, double DIC,
                                                  double Alk, double air, double& H, bool* converged = nullptr) {
    CarbConsts c = col.c;
    c.DIC = DIC * col.conv;
    c.Alk = Alk * col.conv;
    obgc_carbon_options o = g.carbon;
    o.output = OBGC_OUT_PCO2;
    const CarbSolve r = solve_H(o, H, c);
    if (converged) *converged = r.converged;
    H = r.H;
    const double CO2 = c.DIC * (H * H) / (H * H + c.K1 * H + c.K1 * c.K2);
    const double pCO2 = pco2_from_fco2((CO2 / c.K0) * 1e6, col.Tk, 101325.0);
    return col.k_sol * (pCO2 - air);
}

// Every gas-exchange condition of a model in one pass over the surface cells.  The CO2 conditions
// whose carbon-chemistry options equal the first one's (share[q]; the usual case, e.g. one per
// CarbonateSystem replicate) share that column's T/S constants (the equilibrium constants, the
// density conversion, the solubility) and differ only in their water's DIC / Alk, wind and air;
// each condition's Newton solve restarts from its own previous [H+] of the column.
struct GasMulti {
    int n;
    int share[OBGC_MAX_GAS_CONDITIONS];
    obgc_gas_exchange g[OBGC_MAX_GAS_CONDITIONS];
    const void* DIC[OBGC_MAX_GAS_CONDITIONS];
    const void* Alk[OBGC_MAX_GAS_CONDITIONS];
    const void* O2[OBGC_MAX_GAS_CONDITIONS];
    double* flux[OBGC_MAX_GAS_CONDITIONS];
    double* H[OBGC_MAX_GAS_CONDITIONS];
    int* status;   // OBGC_FLAG_NOT_CONVERGED is set here when a pCO2 solve ends unconverged (NULL: none)
};

}  // namespace obgc
