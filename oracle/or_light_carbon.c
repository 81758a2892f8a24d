/*
 * or_light_carbon.c — TEST INFRASTRUCTURE (the oracle).  FP64 restatement of:
 *   src/Light/2band.jl:1-33, multi_band.jl:136-163, compute_euphotic_depth.jl:3-29, Light.jl:45-47
 *   src/Models/CarbonChemistry/{carbon_chemistry.jl, alkalinity_residual.jl,
 *     equilibrium_constants.jl, virial_coefficients.jl, calcite_concentration.jl}
 *   src/Utils/solvers.jl (all four solvers) and the test functions of test/test_solvers.jl:8-25.
 * Seawater density: the reference evaluates SeawaterPolynomials.TEOS10._ρ (SeawaterPolynomials
 * 0.3.x, a third-party package absent here) through teos10_polynomial_approximation
 * (src/Models/seawater_density.jl:33-39).  That is the published 55-term polynomial of Roquet et al.
 * (2015, Ocean Modelling 90:29-43), restated below from the paper's coefficients as a plain sum
 * over its (s, tau, zeta) exponents; the CarbonChemistry doctest digits pin it
 * (carbon_chemistry.jl:55-62).  UNESCO EOS-80 (Millero & Poisson 1981, Millero et al. 1980) and a
 * constant density are the other options.
 */
#include <math.h>
#include <float.h>
#include <string.h>
#include "obgc_oracle.h"

static double jl_min(double a, double b) { return (isnan(a) || isnan(b)) ? NAN : (a < b ? a : b); }
static double jl_sign(double x) { return isnan(x) ? NAN : (x > 0 ? 1.0 : (x < 0 ? -1.0 : 0.0)); }

/* ------------------------------------------------------------------ light ---------- */
/* Light.jl:47 */
double or_default_surface_PAR(double t) { return 100 * fmax(0.0, cos(t * M_PI / (12 * 3600.0))); }

/* 2band.jl:1-33 for one column; zc[0..Nz), zf[0..Nz] (bottom first). */
void or_twoband_column(const obgc_twoband_params* lp, int Nz, const double* zc, const double* zf,
                       const double* P, double PAR0, double* PAR) {
    double kr = lp->water_red_attenuation, kb = lp->water_blue_attenuation;
    double xr = lp->chlorophyll_red_attenuation, xb = lp->chlorophyll_blue_attenuation;
    double er = lp->chlorophyll_red_exponent, eb = lp->chlorophyll_blue_exponent;
    double r = lp->pigment_ratio, Rc = lp->phytoplankton_chlorophyll_ratio;
    int k = Nz - 1;
    double ir = (zf[Nz] - zc[k]) * pow(P[k] * Rc / r, er);
    double ib = (zf[Nz] - zc[k]) * pow(P[k] * Rc / r, eb);
    PAR[k] = PAR0 * (exp(kr * zc[k] - xr * ir) + exp(kb * zc[k] - xb * ib)) / 2;
    for (k = Nz - 2; k >= 0; k--) {
        ir += (zc[k + 1] - zf[k + 1]) * pow(P[k + 1] * Rc / r, er) + (zf[k + 1] - zc[k]) * pow(P[k] * Rc / r, er);
        ib += (zc[k + 1] - zf[k + 1]) * pow(P[k + 1] * Rc / r, eb) + (zf[k + 1] - zc[k]) * pow(P[k] * Rc / r, eb);
        PAR[k] = PAR0 * (exp(kr * zc[k] - xr * ir) + exp(kb * zc[k] - xb * ib)) / 2;
    }
}

/* multi_band.jl:147-163 for one band; `surface` = surface PAR × surface_PAR_division. */
void or_multiband_column(int Nz, const double* zc, double kw, double e, double chi,
                         const double* Chl, double surface, double* PAR) {
    int k = Nz - 1;
    PAR[k] = surface * exp(zc[k] * (kw + chi * pow(Chl[k], e)));
    for (k = Nz - 2; k >= 0; k--) {
        double dz = zc[k] - zc[k + 1];
        PAR[k] = PAR[k + 1] * exp(dz * (kw + chi * pow(Chl[k], e)));
    }
}

/* multi_band.jl:93-104 and numerical_mean :136-140 (findlast(base .<= edge), 1-based in Julia). */
static double numerical_mean(const double* lam, const double* C, int i1, int i2) {
    double s = 0.0;
    for (int n = i1 + 1; n <= i2; n++) s += (C[n] + C[n - 1]) * (lam[n] - lam[n - 1]) / 2;
    return s / (lam[i2] - lam[i1]);
}
void or_multiband_coefficients(int nbands, const double* edges, int nbase, const double* lambda,
                               const double* kw, const double* e, const double* chi,
                               double* okw, double* oe, double* ochi) {
    for (int b = 0; b < nbands; b++) {
        int i1 = -1, i2 = -1;
        for (int n = 0; n < nbase; n++) {
            if (lambda[n] <= edges[2 * b]) i1 = n;
            if (lambda[n] <= edges[2 * b + 1]) i2 = n;
        }
        okw[b] = numerical_mean(lambda, kw, i1, i2);
        oe[b] = numerical_mean(lambda, e, i1, i2);
        ochi[b] = numerical_mean(lambda, chi, i1, i2);
    }
}

/* compute_euphotic_depth.jl:3-29.  PAR_top_halo is PAR[i, j, Nz+1] (the halo above the top
 * cell); zc has Nz+1 entries where zc[-1] (bottom halo centre) is passed as zc_halo via zc[Nz]. */
double or_euphotic_depth_column(int Nz, const double* zc, const double* PAR, double PAR_top_halo,
                                double cutoff) {
    double surface = (PAR[Nz - 1] + PAR_top_halo) / 2;
    double zeu = -INFINITY;
    for (int k = Nz - 2; k >= 0; k--) {
        double Pk = PAR[k];
        if ((Pk <= surface * cutoff) && isinf(zeu)) {
            double Pk1 = PAR[k + 1];
            zeu = zc[k] + (log(surface * cutoff) - log(Pk)) * (zc[k] - zc[k + 1]) / (log(Pk) - log(Pk1));
        }
    }
    return isfinite(zeu) ? zeu : zc[Nz] /* centre of the cell below the bottom */;
}

/* ------------------------------------------------------------------ density ---------- */
/* Roquet et al. (2015): rho = r0(zeta) + sum R_ijk s^i tau^j zeta^k, tau = T / 40,
 * s = sqrt((S_A + 32) / S_u), S_u = 40 x 35.16504 / 35, zeta = -Z / 1e4 with Z the height (m).
 * teos10_polynomial_approximation (seawater_density.jl:33-39) passes T, S_A = S and Z = +10 Pbar. */
static const struct { int i, j, k; double c; } ROQUET[] = {
    {0,0,0, 8.0189615746e+02}, {1,0,0, 8.6672408165e+02}, {2,0,0,-1.7864682637e+03}, {3,0,0, 2.0375295546e+03},
    {4,0,0,-1.2849161071e+03}, {5,0,0, 4.3227585684e+02}, {6,0,0,-6.0579916612e+01},
    {0,1,0, 2.6010145068e+01}, {1,1,0,-6.5281885265e+01}, {2,1,0, 8.1770425108e+01}, {3,1,0,-5.6888046321e+01},
    {4,1,0, 1.7681814114e+01}, {5,1,0,-1.9193502195e+00},
    {0,2,0,-3.7074170417e+01}, {1,2,0, 6.1548258127e+01}, {2,2,0,-6.0362551501e+01}, {3,2,0, 2.9130021253e+01},
    {4,2,0,-5.4723692739e+00},
    {0,3,0, 2.1661789529e+01}, {1,3,0,-3.3449108469e+01}, {2,3,0, 1.9717078466e+01}, {3,3,0,-3.1742946532e+00},
    {0,4,0,-8.3627885467e+00}, {1,4,0, 1.1311538584e+01}, {2,4,0,-5.3563304045e+00},
    {0,5,0, 5.4048723791e-01}, {1,5,0, 4.8169980163e-01}, {0,6,0,-1.9083568888e-01},
    {0,0,1, 1.9681925209e+01}, {1,0,1,-4.2549998214e+01}, {2,0,1, 5.0774768218e+01}, {3,0,1,-3.0938076334e+01},
    {4,0,1, 6.6051753097e+00},
    {0,1,1,-1.3336301113e+01}, {1,1,1,-4.4870114575e+00}, {2,1,1, 5.0042598061e+00}, {3,1,1,-6.5399043664e-01},
    {0,2,1, 6.7080479603e+00}, {1,2,1, 3.5063081279e+00}, {2,2,1,-1.8795372996e+00},
    {0,3,1,-2.4649669534e+00}, {1,3,1,-5.5077101279e-01}, {0,4,1, 5.5927935970e-01},
    {0,0,2, 2.0660924175e+00}, {1,0,2,-4.9527603989e+00}, {2,0,2, 2.5019633244e+00},
    {0,1,2, 2.0564311499e+00}, {1,1,2,-2.1311365518e-01}, {0,2,2,-1.2419983026e+00},
    {0,0,3,-2.3342758797e-02}, {1,0,3,-1.8507636718e-02}, {0,1,3, 3.7969820455e-01},
};
static const double ROQUET_R0[6] = {4.6494977072e+01, -5.2099962525e+00, 2.2601900708e-01, 6.4326772569e-02,
                                    1.5616995503e-02, -1.7243708991e-03};

double or_density_teos10_polynomial(double T, double S, double Pbar) {
    const double Z = 10.0 * Pbar;                 /* seawater_density.jl:34 */
    const double zeta = -Z / 1e4, tau = T / 40.0, s = sqrt((S + 32.0) / (40.0 * 35.16504 / 35.0));
    double rho = 0.0;
    for (int n = 0; n < 6; n++) rho += ROQUET_R0[n] * pow(zeta, n + 1);
    for (size_t q = 0; q < sizeof(ROQUET) / sizeof(ROQUET[0]); q++)
        rho += ROQUET[q].c * pow(s, ROQUET[q].i) * pow(tau, ROQUET[q].j) * pow(zeta, ROQUET[q].k);
    return rho;
}

double or_density(const obgc_carbon_options* o, double T, double S, double Pbar) {
    if (o->density == OBGC_DENSITY_CONSTANT) return o->density_value;
    if (o->density == OBGC_DENSITY_EOS80) return or_density_eos80(T, S, Pbar);
    return or_density_teos10_polynomial(T, S, Pbar);
}

/* UNESCO EOS-80: rho(S, T, p) with p in bar (the reference passes bar and converts 10 m/bar). */
double or_density_eos80(double T, double S, double p) {
    double T2 = T * T, T3 = T2 * T, T4 = T3 * T, T5 = T4 * T;
    double rw = 999.842594 + 6.793952e-2 * T - 9.095290e-3 * T2 + 1.001685e-4 * T3
              - 1.120083e-6 * T4 + 6.536332e-9 * T5;
    double A = 8.24493e-1 - 4.0899e-3 * T + 7.6438e-5 * T2 - 8.2467e-7 * T3 + 5.3875e-9 * T4;
    double B = -5.72466e-3 + 1.0227e-4 * T - 1.6546e-6 * T2;
    double C = 4.8314e-4;
    double S15 = S * sqrt(S);
    double rho0 = rw + A * S + B * S15 + C * S * S;
    if (p == 0.0) return rho0;
    double Kw = 19652.21 + 148.4206 * T - 2.327105 * T2 + 1.360477e-2 * T3 - 5.155288e-5 * T4;
    double Aw = 3.239908 + 1.43713e-3 * T + 1.16092e-4 * T2 - 5.77905e-7 * T3;
    double Bw = 8.50935e-5 - 6.12293e-6 * T + 5.2787e-8 * T2;
    double K0 = Kw + (54.6746 - 0.603459 * T + 1.09987e-2 * T2 - 6.1670e-5 * T3) * S
              + (7.944e-2 + 1.6483e-2 * T - 5.3009e-4 * T2) * S15;
    double Ap = Aw + (2.2838e-3 - 1.0981e-5 * T - 1.6078e-6 * T2) * S + 1.91075e-4 * S15;
    double Bp = Bw + (-9.9348e-7 + 2.0816e-8 * T + 9.1697e-10 * T2) * S;
    double K = K0 + Ap * p + Bp * p * p;
    return rho0 / (1 - p / K);
}

/* ------------------------------------------------------------------ constants ---------- */
/* PressureCorrection (equilibrium_constants.jl:11-40): a0 a1 a2 b0 b1 for each constant. */
static const double PC[OR_NUM_K][5] = {
    /* K0  */ {0, 0, 0, 0, 0},
    /* K1  */ {-25.50, 0.1271, 0.0, -0.00308, 0.0000877},
    /* K2  */ {-15.82, -0.0219, 0.0, 0.00113, -0.0001475},
    /* KB  */ {-29.48, 0.1622, -0.0026080, -0.00284, 0.0},
    /* KW  */ {-20.02, 0.1119, -0.001409, -0.00513, 0.0000794},
    /* KS  */ {-18.03, 0.0466, 0.000316, -0.00453, 0.00009},
    /* KF  */ {-9.78, -0.0090, -0.000942, -0.00391, 0.000054},
    /* KP1 */ {-14.51, 0.1211, -0.000321, -0.00267, 0.0000427},
    /* KP2 */ {-23.12, 0.1758, -0.002647, -0.00515, 0.00009},
    /* KP3 */ {-26.57, 0.2020, -0.0030420, -0.00408, 0.0000714},
    /* KSi */ {0, 0, 0, 0, 0},
    /* KSP calcite   */ {-48.76, 0.5304, -0.0, -0.01176, 0.0003692},
    /* KSP aragonite */ {-45.96, 0.5304, -0.0, -0.01176, 0.0003692},
};

double or_pressure_correction(int which, double Tk, double P) {
    const double* c = PC[which];
    double R = 83.14472;
    double Tc = Tk - 273.15;
    double dV = c[0] + c[1] * Tc + c[2] * (Tc * Tc);
    double dk = c[3] + c[4] * Tc;
    double RT = R * Tk;
    return exp((-dV + 0.5 * dk * P) * P / RT);
}

static double ionic_strength(double S) { return 19.924 * S / (1000.0 + -1.005 * S); }

static double KS_value(double T, double S, double Is) {
    return exp(141.328 + -4276.1 / T + -23.093 * log(T)
               + (324.57 + -13856.0 / T + -47.986 * log(T)) * sqrt(Is)
               + (-771.54 + 35474.0 / T + 114.723 * log(T)) * Is
               + -2698.0 * pow(Is, 1.5) / T
               + 1776.0 * (Is * Is) / T
               + log(1 + -0.001005 * S));
}

double or_equilibrium_constant(int which, double T, double S, int has_P, double P) {
    double pc = has_P ? or_pressure_correction(which, T, P) : 1.0;
    double v;
    switch (which) {
        case OR_K0:  /* :65-80 */
            return exp(-60.2409 + (93.4517 * 100) / T + 23.3585 * (log(T) - log(100.0)) + 0.0 * pow(T, 2.0)
                       + (0.023517 + (-0.023656 / 100) * T + (0.0047036 / 10000) * pow(T, 2.0)) * S);
        case OR_K1:  /* :103-126 */
            v = pow(10.0, 61.2172 + -3633.86 / T + -9.67770 * log(T) + 0.011555 * S + -0.0001152 * (S * S));
            return pc * v;
        case OR_K2:  /* :149-172 */
            v = pow(10.0, -25.9290 + -471.78 / T + 0.01781 * S + -0.0001122 * (S * S) + 3.16967 * log(T));
            return pc * v;
        case OR_KB: {/* :202-250 */
            double sS = sqrt(S);
            v = exp(148.0248 + (-8966.90 + -2890.53 * sS + -77.942 * S + 1.728 * pow(S, 1.5) + -0.0996 * pow(S, 2.0)) / T
                    + 137.1942 * sS + 1.62142 * S + (-24.4344 + -25.085 * sS + -0.2474 * S) * log(T)
                    + 0.053105 * sS * T);
            return pc * v;
        }
        case OR_KW:  /* :279-313 */
            v = exp(148.9652 + -13847.26 / T + -23.6521 * log(T)
                    + (-5.977 + 118.67 / T + 1.0495 * log(T)) * sqrt(S) + -0.01615 * S);
            return pc * v;
        case OR_KS:  /* :366-419 */
            return pc * KS_value(T, S, ionic_strength(S));
        case OR_KF: {/* :451-487 (log_S = log_S_KS = 0) */
            double Is = ionic_strength(S);
            double KS = KS_value(T, S, Is);
            v = exp(-9.68 + 874.0 / T + 0.111 * sqrt(S) + log(1 + 0.0 * S) + log(1 + 0.0 * S / KS));
            return pc * v;
        }
        case OR_KP1: /* :511-651 */
            v = exp(115.525 + -4576.752 / T + -18.453 * log(T) + (0.69171 + -106.736 / T) * sqrt(S)
                    + (-0.01844 + -0.65643 / T) * S);
            return pc * v;
        case OR_KP2:
            v = exp(172.0883 + -8814.715 / T + -27.927 * log(T) + (1.3566 + -160.340 / T) * sqrt(S)
                    + (-0.05778 + 0.37335 / T) * S);
            return pc * v;
        case OR_KP3:
            v = exp(-18.141 + -3070.75 / T + 0.0 * log(T) + (2.81197 + 17.27039 / T) * sqrt(S)
                    + (-0.09984 + -44.99486 / T) * S);
            return pc * v;
        case OR_KSI: {/* :674-713 (no pressure correction) */
            double Is = ionic_strength(S);
            return exp(117.385 + -8904.2 / T + -19.334 * log(T) + (3.5913 + -458.79 / T) * sqrt(Is)
                       + (-1.5998 + 188.74 / T) * Is + (0.07871 + -12.1652 / T) * (Is * Is)
                       + log(1 + -0.001005 * S));
        }
        case OR_KSP_CALCITE: case OR_KSP_ARAGONITE: {/* :740-850, log10(T) kept as in :758 */
            int c = which == OR_KSP_CALCITE;
            double tc = c ? -171.9065 : -171.945, tT = -0.077993, tiT = c ? 2839.319 : 2903.293, tl = 71.595;
            double ss = c ? -0.77712 : -0.068393, sT = c ? 0.0028426 : 0.0017276, siT = c ? 178.34 : 88.135;
            double sS = c ? -0.07711 : -0.10018, sS3 = c ? 0.0041249 : 0.0059415;
            double lnK_therm = tc + tT * T + tiT / T + tl * log10(T);
            double lnK_sea = (ss + sT * T + siT / T) * sqrt(S) + sS * S + sS3 * pow(S, 1.5);
            return pc * pow(10.0, lnK_therm + lnK_sea);
        }
    }
    return NAN;
}

/* virial_coefficients.jl:1-17 */
double or_first_virial(double Tk) {
    return (-1636.75 + 12.0408 * Tk + (-3.27957 * 1e-2) * (Tk * Tk) + (3.16528 * 1e-5) * (Tk * Tk * Tk)) * 1e-6;
}
double or_cross_virial(double Tk) { return (57.7 + -0.118 * Tk) * 1e-6; }

/* ------------------------------------------------------------------ alkalinity ---------- */
typedef struct {
    double DIC, Alk, boron, sulfate, fluoride, silicate, phosphate;
    double K1, K2, KB, KW, KS, KF, KP1, KP2, KP3, KSi;
} carb_params;

/* alkalinity_residual.jl:18-75 */
static double alk_residual(double H, const carb_params* p) {
    double cd = H * H + p->K1 * H + p->K1 * p->K2;
    double pd = H * H * H + p->KP1 * (H * H) + p->KP1 * p->KP2 * H + p->KP1 * p->KP2 * p->KP3;
    double sd = 1 + p->sulfate / p->KS;
    double bicarbonate = p->K1 * H * p->DIC / cd;
    double carbonate = 2 * p->DIC * p->K1 * p->K2 / cd;
    double borate = p->boron / (1 + H / p->KB);
    double hydroxide = p->KW / H;
    double hydrogen_phosphate = p->phosphate * p->KP1 * p->KP2 * H / pd;
    double phosphate = 2 * p->phosphate * p->KP1 * p->KP2 * p->KP3 / pd;
    double silicate = p->silicate / (1 + H / p->KSi);
    double free_hydrogen = -H / sd;
    double hydrogen_sulfate = -p->sulfate / (1 + p->KS / H * sd);
    double hydrogen_fluoride = -p->fluoride / (1 + p->KF / H);
    double phosphoric_acid = -p->phosphate * (H * H * H) / pd;
    return bicarbonate + carbonate + borate + hydroxide + hydrogen_phosphate + phosphate + silicate
         + free_hydrogen + hydrogen_sulfate + hydrogen_fluoride + phosphoric_acid - p->Alk;
}
static double alk_residual_dH(double H, const carb_params* p) {
    double cd = H * H + p->K1 * H + p->K1 * p->K2;
    double pd = H * H * H + p->KP1 * (H * H) + p->KP1 * p->KP2 * H + p->KP1 * p->KP2 * p->KP3;
    double sd = 1 + p->sulfate / p->KS;
    double dcd = 2 * H + p->K1;
    double dpd = 3 * (H * H) + 2 * p->KP1 * H + p->KP1 * p->KP2;
    double dsd = 0;
    double a = p->K1 * p->DIC * (p->K1 * p->K2 - H * H) / (cd * cd);
    double b = -dcd * 2 * p->DIC * p->K1 * p->K2 / (cd * cd);
    double q = 1 + H / p->KB;
    double c = -p->boron / (q * q) / p->KB;
    double d = -p->KW / (H * H);
    double e = p->phosphate * p->KP1 * p->KP2 / pd - dpd * p->phosphate * p->KP1 * p->KP2 * H / (pd * pd);
    double f = -dpd * 2 * p->phosphate * p->KP1 * p->KP2 * p->KP3 / (pd * pd);
    double qs = 1 + H / p->KSi;
    double g = -p->silicate / (qs * qs) / p->KSi;
    double h = -1 / sd;
    double qh = 1 + p->KS / H * sd;
    double i = p->sulfate / (qh * qh) * (p->KS / H * dsd - p->KS / (H * H) * sd);
    double qf = 1 + p->KF / H;
    double j = -p->fluoride / (qf * qf) * p->KF / (H * H);
    double k = -3 * p->phosphate * (H * H) / pd - dpd * p->phosphate * (H * H * H) / (pd * pd);
    return a + b + c + d + e + f + g + h + i + j + k;
}

/* solvers.jl:123-141 with lower bound L (upper = nothing) */
static double bounded_lambda_lower(double x, double L, double d) {
    double lb = (x - L) / d;
    lb = lb < 0 ? 1.0 : lb;
    return jl_min(1.0, lb);
}

/* DampedNewtonRaphsonSolver (solvers.jl:81-121) on the alkalinity residual, bounds (0, nothing). */
static double damped_newton_H(const obgc_carbon_options* o, double x0, const carb_params* p, int* iters) {
    double x = x0;
    int N = 0;
    double lm = o->min_damping, c = o->armijo_constant;
    double fx = alk_residual(x, p);
    while ((fabs(fx) > o->atol) & (N < o->max_iters)) {
        double d = fx / alk_residual_dH(x, p);
        double lam = bounded_lambda_lower(x, 0.0, d);
        double fnew = alk_residual(x - lam * d, p);
        while ((fabs(fnew) >= fabs(fx) - c * lam * fx * jl_sign(fx)) & (lam > lm)) {
            lam *= o->damping;
            fnew = alk_residual(x - lam * d, p);
        }
        x -= lam * d;
        N += 1;
        fx = fnew;
    }
    if (iters) *iters = N;
    return x;
}

int or_carbon_default_options(obgc_carbon_options* o) {
    memset(o, 0, sizeof(*o));
    o->output = OBGC_OUT_FCO2;
    o->density = OBGC_DENSITY_TEOS10_POLYNOMIAL;
    o->max_iters = 100;
    o->initial_pH_guess = 8.0;
    o->atol = 1e-20;
    o->damping = 0.5;
    o->armijo_constant = 0.5;
    o->min_damping = pow(0.5, 10);
    o->calcium_ion_per_salinity = 0.0103 / 35;
    return 0;
}

/* carbon_chemistry.jl:111-218 and calcite_concentration.jl:1-80. */
int or_carbon_chemistry(const obgc_carbon_options* o, double DIC, double Alk, double T, double S,
                        double silicate, double phosphate, double P, double pH, double* out, int* iters) {
    int carbonate_path = (o->output == OBGC_OUT_CARBONATE || o->output == OBGC_OUT_OMEGA_CALCITE);
    int hasP = o->has_pressure;
    double T_c = T;
    /* density at P (or 1 bar for the pCO2 functor, 0 bar for carbonate_concentration) */
    double Pd = hasP ? P : (carbonate_path ? 0.0 : 1.0);
    double rho = or_density(o, T, S, Pd);
    double boron = 0.000232 / 10.811 * S / 1.80655;
    double sulfate = 0.14 / 96.06 * S / 1.80655;
    double fluoride = 0.000067 / 18.9984 * S / 1.80655;
    T += 273.15;
    Alk *= 1e-3 / rho;
    DIC *= 1e-3 / rho;
    phosphate *= 1e-3 / rho;
    silicate *= 1e-3 / rho;
    double Is = ionic_strength(S);
    carb_params p;
    p.DIC = DIC; p.Alk = Alk; p.boron = boron; p.sulfate = sulfate; p.fluoride = fluoride;
    p.silicate = silicate; p.phosphate = phosphate;
    p.K1 = or_equilibrium_constant(OR_K1, T, S, hasP, P);
    p.K2 = or_equilibrium_constant(OR_K2, T, S, hasP, P);
    p.KB = or_equilibrium_constant(OR_KB, T, S, hasP, P);
    p.KW = or_equilibrium_constant(OR_KW, T, S, hasP, P);
    p.KS = (hasP ? or_pressure_correction(OR_KS, T, P) : 1.0) * KS_value(T, S, Is);
    p.KF = or_equilibrium_constant(OR_KF, T, S, hasP, P);
    p.KP1 = or_equilibrium_constant(OR_KP1, T, S, hasP, P);
    p.KP2 = or_equilibrium_constant(OR_KP2, T, S, hasP, P);
    p.KP3 = or_equilibrium_constant(OR_KP3, T, S, hasP, P);
    p.KSi = or_equilibrium_constant(OR_KSI, T, S, 0, 0);
    double H;
    int it = 0;
    if (o->ph_given) H = pow(10.0, -pH);
    else H = damped_newton_H(o, pow(10.0, -o->initial_pH_guess), &p, &it);
    if (iters) *iters = it;
    if (carbonate_path) {
        double d1 = H * (H + p.K1);
        double d2 = 1.0 + p.K1 * p.K2 / d1;
        double co3 = DIC * p.K1 * p.K2 / d1 / d2;
        if (o->output == OBGC_OUT_CARBONATE) { *out = co3; return 0; }
        double KSP = or_equilibrium_constant(o->saturation_mineral == 1 ? OR_KSP_ARAGONITE : OR_KSP_CALCITE, T_c + 273.15, S,
                                             hasP, P);
        double Ca = 0.0103 * S / 35;
        *out = Ca * co3 / KSP;
        return 0;
    }
    double K0 = or_equilibrium_constant(OR_K0, T, S, 0, 0);
    double CO2 = DIC * (H * H) / (H * H + p.K1 * H + p.K1 * p.K2);
    double fCO2 = (CO2 / K0) * 1e6;
    switch (o->output) {
        case OBGC_OUT_FCO2: *out = fCO2; return 0;
        case OBGC_OUT_H: *out = H; return 0;
        case OBGC_OUT_PH_FREE: *out = -log10(H); return 0;
        case OBGC_OUT_PCO2: {
            double Pp = (hasP ? P : 1.0) * 101325;
            double B = or_first_virial(T), dl = or_cross_virial(T);
            double f = fCO2 * 0.09807;
            double phi = 1.0;
            double x = f / (phi * Pp);
            for (int n = 0; n < 3; n++) {
                phi = exp((B + 2.0 * pow(1.0 - x, 2.0) * dl) * Pp / (8.31446261815324 * T));
                x = f / (phi * Pp);
            }
            double pCO2 = f / phi;
            *out = pCO2 / 0.09807;
            return 0;
        }
        case OBGC_OUT_PH_TOTAL: {
            double KS = p.KS;
            double HSO4 = sulfate / (1 + KS / H);
            *out = -log10(H + HSO4);
            return 0;
        }
        case OBGC_OUT_PH_SWS: {
            double KS = p.KS;
            double HSO4 = sulfate / (1 + KS / H);
            double KF = p.KF;
            double HF = fluoride / (1 + KF / H);
            *out = -log10(H + HSO4 + HF);
            return 0;
        }
    }
    return -1;
}

void or_carbon_chemistry_batch(const obgc_carbon_options* o, int64_t n, const double* DIC,
                               const double* Alk, const double* T, const double* S,
                               const double* Si, const double* PO4, const double* P,
                               const double* pH, double* out, int nthreads) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int64_t i = 0; i < n; i++)
        or_carbon_chemistry(o, DIC[i], Alk[i], T[i], S[i], Si ? Si[i] : 0.0, PO4 ? PO4[i] : 0.0,
                            P ? P[i] : 0.0, pH ? pH[i] : 0.0, &out[i], NULL);
}

/* ------------------------------------------------------------------ solvers ---------- */
/* test/test_solvers.jl:8-25 */
static double tf(int id, double x, double pa, double pb) {
    switch (id) {
        case 1: return tanh(x);
        case 2: return x * x - 2;
        case 3: return exp(x) - 1000;
        case 4: return 1 / (1 + x * x) - 0.5;
        default: return pa * (x * x) + pb;
    }
}
static double tfp(int id, double x, double pa, double pb) {
    (void)pb;
    switch (id) {
        case 1: { double s = 1 / cosh(x); return s * s; }
        case 2: return 2 * x;
        case 3: return exp(x);
        case 4: { double q = 1 + x * x; return -2 * x / (q * q); }
        default: return 2 * pa * x;
    }
}
/* solvers.jl:70-75 */
static void bisection_step(double xp, double xm, double x, int id, double pa, double pb, double* nm, double* np) {
    double fx = tf(id, x, pa, pb);
    *nm = ((jl_sign(tf(id, xm, pa, pb)) == jl_sign(fx)) | (fx == 0)) ? x : xm;
    *np = ((jl_sign(tf(id, xp, pa, pb)) == jl_sign(fx)) | (fx == 0)) ? x : xp;
}

double or_solve_test_function(int solver, int id, double x0, double x1, double damping, double pa, double pb) {
    if (solver == OR_SOLVER_NEWTON) {           /* solvers.jl:1-22, max_iters 1000, atol 1e-10 */
        double x = x0; int N = 0;
        double fx = tf(id, x, pa, pb);
        while ((fabs(fx) > 1e-10) & (N < 1000)) {
            fx = tf(id, x, pa, pb);
            x -= fx / tfp(id, x, pa, pb);
            N += 1;
        }
        return x;
    }
    if (solver == OR_SOLVER_NEWTON_SAFE) {      /* solvers.jl:24-48, max_iters 100 */
        double xm = fmin(x0, x1), xp = fmax(x0, x1);
        double xn = (xm + xp) / 2; int N = 0;
        while ((fabs(tf(id, (xm + xp) / 2, pa, pb)) > 1e-10) & (N < 100)) {
            xn = (xm + xp) / 2;
            double xn1 = xn - tf(id, xn, pa, pb) / tfp(id, xn, pa, pb);
            double nm, np;
            bisection_step(xp, xm, ((xm < xn1) && (xn1 < xp)) ? xn1 : xn, id, pa, pb, &nm, &np);
            xm = nm; xp = np;
            xn = (xm + xp) / 2;
            N += 1;
        }
        return xn;
    }
    if (solver == OR_SOLVER_BISECTION) {        /* solvers.jl:50-68 */
        double xm = x0, xp = x1;
        double xn = (xm + xp) / 2; int N = 0;
        while ((fabs(tf(id, xn, pa, pb)) > 1e-10) & (N < 100)) {
            double nm, np;
            bisection_step(xp, xm, xn, id, pa, pb, &nm, &np);
            xm = nm; xp = np;
            xn = (xm + xp) / 2;
            N += 1;
        }
        return xn;
    }
    /* DampedNewtonRaphsonSolver, no bounds (solvers.jl:81-121) */
    double x = x0; int N = 0;
    double lm = pow(damping, 10), c = 0.5;
    double fx = tf(id, x, pa, pb);
    while ((fabs(fx) > 1e-20) & (N < 100)) {
        double d = fx / tfp(id, x, pa, pb);
        double lam = 1.0;
        double fnew = tf(id, x - lam * d, pa, pb);
        while ((fabs(fnew) >= fabs(fx) - c * lam * fx * jl_sign(fx)) & (lam > lm)) {
            lam *= damping;
            fnew = tf(id, x - lam * d, pa, pb);
        }
        x -= lam * d;
        N += 1;
        fx = fnew;
    }
    return x;
}
