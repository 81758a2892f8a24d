/* or_gas.c — oracle (test infrastructure): CPU restatement of OceanBioME's air-sea gas exchange
 * (src/Models/GasExchange), FP64.  Not part of the product; the tests compare the CUDA path with it.
 *
 *   GasExchange functor            gas_exchange.jl:26-39        flux = k (C_water - C_air)
 *   SchmidtScaledTransferVelocity  gas_transfer_velocity.jl:25-31  k = k660(u10) / sqrt(Sc(T)/660) * sol(T, S)
 *   Ho06 k660                      gas_transfer_velocity.jl:53-59  0.266 / hour / 100 * u^2
 *   Schmidt numbers (Wanninkhof 2014)  schmidt_number.jl:1-16
 *   CO2 water concentration        carbon_dioxide_concentration.jl:48-60 (pCO2, silicate = phosphate = 0)
 *   CO2 solubility                 gas_solubility.jl:58-64  K0(T + 273.15, S) * rho(T, S) / 1000
 *   O2 air concentration           gas_solubility.jl:1-25 (PartiallySolubleGas), :28-56 (Wanninkhof92Solubility)
 *   defaults                       GasExchange.jl:96-146
 * The O2 solubility is evaluated as the reference writes it: the salinity term uses B2 for both the
 * linear and the quadratic coefficient (gas_solubility.jl:47), so B3 is unused.
 */
#include <math.h>
#include <string.h>
#include "obgc_oracle.h"

static const double HOUR = 3600.0;

int or_gas_exchange_defaults(int gas, obgc_gas_exchange* g) {
    memset(g, 0, sizeof(*g));
    g->gas = gas;
    g->k660[2] = 0.266 / HOUR / 100;          /* Ho06 */
    g->wind_speed = 2.0;
    or_carbon_default_options(&g->carbon);
    g->carbon.output = OBGC_OUT_PCO2;
    if (gas == OBGC_GAS_CO2) {
        const double s[5] = {2116.8, -136.25, 4.7353, -0.092307, 0.0007555};
        memcpy(g->schmidt, s, sizeof(s));
        g->air_concentration = 413.0;
    } else if (gas == OBGC_GAS_O2) {
        const double s[5] = {1920.4, -135.6, 5.2122, -0.10939, 0.00093777};
        const double a[6] = {-58.3877, 85.8079, 23.8439, -0.034892, 0.015578, -0.0019387};
        memcpy(g->schmidt, s, sizeof(s));
        memcpy(g->o2_solubility, a, sizeof(a));
        g->air_concentration = 9352.7;
    } else {
        return -1;
    }
    return 0;
}

/* PolynomialParameterisation{4} (generic_parameterisations.jl:34-35) */
double or_schmidt_number(const double* c, double T) {
    return c[0] + c[1] * T + c[2] * pow(T, 2.0) + c[3] * pow(T, 3.0) + c[4] * pow(T, 4.0);
}

/* PolynomialParameterisation{2} / {3} in u10 */
double or_transfer_velocity_660(const double* c, double u) {
    return c[0] + c[1] * u + c[2] * pow(u, 2.0) + c[3] * pow(u, 3.0);
}

/* Wanninkhof92Solubility as the reference evaluates it (gas_solubility.jl:40-50) */
double or_o2_solubility(const double* A, double T, double S) {
    const double Tk = T + 273.15;
    const double Tk_100 = Tk / 100.0;
    const double beta = exp(A[0] + A[1] / Tk_100 + A[2] * log(Tk_100) + S * (A[3] + A[4] * Tk_100 + A[4] * pow(Tk_100, 2.0)));
    return beta / Tk;
}

double or_gas_exchange_flux(const obgc_gas_exchange* g, double T, double S, double DIC, double Alk, double O2,
                            double u10, double air) {
    const double k660 = or_transfer_velocity_660(g->k660, u10);
    const double Sc = or_schmidt_number(g->schmidt, T);
    if (g->gas == OBGC_GAS_CO2) {
        /* the carbon chemistry's density function at zero pressure (gas_solubility.jl:58-65) */
        const double solubility = or_equilibrium_constant(OR_K0, T + 273.15, S, 0, 0.0) * or_density(&g->carbon, T, S, 0.0) / 1000.0;
        const double k = k660 / sqrt(Sc / 660.0) * solubility;
        obgc_carbon_options o = g->carbon;
        o.output = OBGC_OUT_PCO2;
        o.ph_given = 0;
        double pCO2 = 0.0;
        or_carbon_chemistry(&o, DIC, Alk, T, S, 0.0, 0.0, 0.0, 0.0, &pCO2, NULL);
        return k * (pCO2 - air);
    }
    const double k = k660 / sqrt(Sc / 660.0);
    return k * (O2 - air * or_o2_solubility(g->o2_solubility, T, S));
}
