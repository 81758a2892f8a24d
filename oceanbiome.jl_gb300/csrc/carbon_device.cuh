// carbon_device.cuh — the CarbonChemistry functor in FP64 (host and device).
//
// Follows src/Models/CarbonChemistry/carbon_chemistry.jl:111-218 (unit conversion, constants,
// solve, outputs), alkalinity_residual.jl:18-75, equilibrium_constants.jl (coefficients below are
// the reference's defaults: Weiss 1974 K0, Lueker et al. 2000 K1/K2, Dickson 1990 KB/KS, Millero
// 1995 KW/KP/KSi, Perez & Fraga 1987 KF, Millero 2007 KSP and pressure corrections),
// virial_coefficients.jl and calcite_concentration.jl.
//
// The root solve is the reference's DampedNewtonRaphsonSolver (src/Utils/solvers.jl:81-121:
// Armijo backtracking, damping 0.5, lower bound H >= 0, |residual| <= atol) with two additions:
// it also stops once the Newton step no longer changes H at FP64 resolution (the reference keeps
// backtracking at that point until max_iters), and a cell that still has not converged is finished
// by bisection on a bracket of the monotone residual (the bisection guard).
#pragma once
#include "obgc_common.cuh"

namespace obgc {

// Seawater density of the default CarbonChemistry, teos10_polynomial_approximation
// (src/Models/seawater_density.jl:33-39): the 55-term TEOS-10 polynomial of Roquet, Madec,
// McDougall & Barker (2015, Ocean Modelling 90:29-43) for in-situ density as a function of
// conservative temperature, absolute salinity and depth, rho = r0(zeta) + rho'(tau, s, zeta) with
// tau = T / 40, s = sqrt((S + 32) / (40 x 35.16504 / 35)) and zeta = -Z / 1e4.  The reference feeds
// it T as the conservative temperature, S as the absolute salinity and Z = +10 m per bar of P
// (positive: the polynomial's Z is a height, so zeta = -P / 1000 places the cell above the sea
// surface); this function does the same.  Horner form in zeta, then tau, then s.
__host__ __device__ inline double density_teos10_poly(double T, double S, double Pbar) {
    const double z = -(10.0 * Pbar) * 1e-4;
    const double t = T * 0.025;
    const double s = sqrt((S + 32.0) * (35.0 / (40.0 * 35.16504)));
    // zeta^0: coefficients of tau^0 .. tau^6, each a polynomial in s
    const double a0 = (((((-6.0579916612e+01 * s + 4.3227585684e+02) * s - 1.2849161071e+03) * s + 2.0375295546e+03) * s -
                        1.7864682637e+03) * s + 8.6672408165e+02) * s + 8.0189615746e+02;
    const double a1 = ((((-1.9193502195 * s + 1.7681814114e+01) * s - 5.6888046321e+01) * s + 8.1770425108e+01) * s -
                       6.5281885265e+01) * s + 2.6010145068e+01;
    const double a2 = (((-5.4723692739 * s + 2.9130021253e+01) * s - 6.0362551501e+01) * s + 6.1548258127e+01) * s -
                      3.7074170417e+01;
    const double a3 = ((-3.1742946532 * s + 1.9717078466e+01) * s - 3.3449108469e+01) * s + 2.1661789529e+01;
    const double a4 = (-5.3563304045 * s + 1.1311538584e+01) * s - 8.3627885467;
    const double a5 = 4.8169980163e-01 * s + 5.4048723791e-01;
    const double p0 = (((((-1.9083568888e-01 * t + a5) * t + a4) * t + a3) * t + a2) * t + a1) * t + a0;
    // zeta^1
    const double b0 = (((6.6051753097 * s - 3.0938076334e+01) * s + 5.0774768218e+01) * s - 4.2549998214e+01) * s +
                      1.9681925209e+01;
    const double b1 = ((-6.5399043664e-01 * s + 5.0042598061) * s - 4.4870114575) * s - 1.3336301113e+01;
    const double b2 = (-1.8795372996 * s + 3.5063081279) * s + 6.7080479603;
    const double b3 = -5.5077101279e-01 * s - 2.4649669534;
    const double p1 = (((5.5927935970e-01 * t + b3) * t + b2) * t + b1) * t + b0;
    // zeta^2 and zeta^3
    const double p2 = (-1.2419983026 * t + (-2.1311365518e-01 * s + 2.0564311499)) * t +
                      ((2.5019633244 * s - 4.9527603989) * s + 2.0660924175);
    const double p3 = 3.7969820455e-01 * t - 1.8507636718e-02 * s - 2.3342758797e-02;
    // reference profile r0(zeta)
    const double r0 = z * (4.6494977072e+01 + z * (-5.2099962525 + z * (2.2601900708e-01 + z * (6.4326772569e-02 +
                      z * (1.5616995503e-02 + z * -1.7243708991e-03)))));
    return r0 + (p0 + z * (p1 + z * (p2 + z * p3)));
}

// UNESCO EOS-80 (Millero & Poisson 1981; Millero et al. 1980 secant bulk modulus), p in bar: the
// OBGC_DENSITY_EOS80 option.
__host__ __device__ inline double density_eos80(double T, double S, double p) {
    const double T2 = T * T, T3 = T2 * T, T4 = T3 * T, T5 = T4 * T;
    const double rw = 999.842594 + 6.793952e-2 * T - 9.095290e-3 * T2 + 1.001685e-4 * T3 - 1.120083e-6 * T4 +
                      6.536332e-9 * T5;
    const double A = 8.24493e-1 - 4.0899e-3 * T + 7.6438e-5 * T2 - 8.2467e-7 * T3 + 5.3875e-9 * T4;
    const double B = -5.72466e-3 + 1.0227e-4 * T - 1.6546e-6 * T2;
    const double S15 = S * sqrt(S);
    const double rho0 = rw + A * S + B * S15 + 4.8314e-4 * S * S;
    if (p == 0.0) return rho0;
    const double Kw = 19652.21 + 148.4206 * T - 2.327105 * T2 + 1.360477e-2 * T3 - 5.155288e-5 * T4;
    const double Aw = 3.239908 + 1.43713e-3 * T + 1.16092e-4 * T2 - 5.77905e-7 * T3;
    const double Bw = 8.50935e-5 - 6.12293e-6 * T + 5.2787e-8 * T2;
    const double K0 = Kw + (54.6746 - 0.603459 * T + 1.09987e-2 * T2 - 6.1670e-5 * T3) * S +
                      (7.944e-2 + 1.6483e-2 * T - 5.3009e-4 * T2) * S15;
    const double Ap = Aw + (2.2838e-3 - 1.0981e-5 * T - 1.6078e-6 * T2) * S + 1.91075e-4 * S15;
    const double Bp = Bw + (-9.9348e-7 + 2.0816e-8 * T + 9.1697e-10 * T2) * S;
    return rho0 / (1 - p / (K0 + Ap * p + Bp * p * p));
}

// The density a CarbonChemistry's options select, at P bar.
__host__ __device__ inline double seawater_density(const obgc_carbon_options& o, double T, double S, double Pbar) {
    return o.density == OBGC_DENSITY_CONSTANT ? o.density_value
         : o.density == OBGC_DENSITY_EOS80   ? density_eos80(T, S, Pbar)
                                              : density_teos10_poly(T, S, Pbar);
}

// PressureCorrection (equilibrium_constants.jl:11-40): the log of the factor, so that a constant
// and its correction take one exp between them.
// iRT = 1 / (R Tk), shared by every constant of a cell.
__host__ __device__ inline double pressure_log(double a0, double a1, double a2, double b0, double b1, double Tk, double P,
                                               double iRT) {
    const double Tc = Tk - 273.15;
    const double dV = a0 + a1 * Tc + a2 * (Tc * Tc);
    const double dk = b0 + b1 * Tc;
    return (-dV + 0.5 * dk * P) * P * iRT;
}

// K0 = [CO2*(aq)] / f(CO2): Weiss (1974) (equilibrium_constants.jl:65-80); lT = log(Tk), iT = 1/Tk.
__host__ __device__ inline double weiss_k0(double Tk, double S, double lT, double iT) {
    return exp(-60.2409 + (93.4517 * 100) * iT + 23.3585 * (lT - 4.605170185988092) +
               (0.023517 + (-0.023656 / 100) * Tk + (0.0047036 / 10000) * (Tk * Tk)) * S);
}

struct CarbConsts {
    double DIC, Alk, boron, sulfate, fluoride, silicate, phosphate;
    double K1, K2, KB, KW, KS, KF, KP1, KP2, KP3, KSi, K0;
    double lT, iT, sS, iRT;      // log(Tk), 1/Tk, sqrt(S), 1/(R Tk), kept for the outputs
    // H-independent pieces of the residual (prepare_residual)
    double sd, isd, iKB, iKSi, KSsd, K1K2, KP12, KP123, PKK;
};

__host__ __device__ inline void prepare_residual(CarbConsts& p) {
    p.sd = 1 + p.sulfate / p.KS;
    p.isd = 1.0 / p.sd;
    p.iKB = 1.0 / p.KB;
    p.iKSi = p.KSi != 0.0 ? 1.0 / p.KSi : 0.0;   // KSi is left at zero without silicate
    p.KSsd = p.KS * p.sd;
    p.K1K2 = p.K1 * p.K2;
    p.KP12 = p.KP1 * p.KP2;
    p.KP123 = p.KP12 * p.KP3;
    p.PKK = p.phosphate * p.KP12;
}

// The equilibrium constants at (Tk, S[, P]) with logs and roots shared between them.  A constant
// whose species is absent (phosphate or silicate zero) or whose output is not asked for (K0 outside
// fCO2 / pCO2) is left at zero: every term it enters is then multiplied by that zero concentration.
__host__ __device__ inline void equilibrium_constants(double Tk, double S, bool hasP, double P, bool need_K0, CarbConsts& c) {
    const double lT = log(Tk), iT = 1.0 / Tk, sS = sqrt(S);
    const double iRT = iT * (1.0 / 83.14472);
    c.lT = lT; c.iT = iT; c.sS = sS; c.iRT = iRT;
    const double Is = 19.924 * S / (1000.0 + -1.005 * S);
    const double sIs = sqrt(Is);
    const double LN10 = 2.302585092994046;
    const double pK1 = hasP ? pressure_log(-25.50, 0.1271, 0.0, -0.00308, 0.0000877, Tk, P, iRT) : 0.0;
    const double pK2 = hasP ? pressure_log(-15.82, -0.0219, 0.0, 0.00113, -0.0001475, Tk, P, iRT) : 0.0;
    const double pKB = hasP ? pressure_log(-29.48, 0.1622, -0.0026080, -0.00284, 0.0, Tk, P, iRT) : 0.0;
    const double pKW = hasP ? pressure_log(-20.02, 0.1119, -0.001409, -0.00513, 0.0000794, Tk, P, iRT) : 0.0;
    const double pKS = hasP ? pressure_log(-18.03, 0.0466, 0.000316, -0.00453, 0.00009, Tk, P, iRT) : 0.0;
    const double pKF = hasP ? pressure_log(-9.78, -0.0090, -0.000942, -0.00391, 0.000054, Tk, P, iRT) : 0.0;
    const double pP1 = hasP ? pressure_log(-14.51, 0.1211, -0.000321, -0.00267, 0.0000427, Tk, P, iRT) : 0.0;
    const double pP2 = hasP ? pressure_log(-23.12, 0.1758, -0.002647, -0.00515, 0.00009, Tk, P, iRT) : 0.0;
    const double pP3 = hasP ? pressure_log(-26.57, 0.2020, -0.0030420, -0.00408, 0.0000714, Tk, P, iRT) : 0.0;
    // K1, K2: Lueker et al. (2000), log10 form (:103-172)
    c.K1 = exp(LN10 * (61.2172 + -3633.86 * iT + -9.67770 * lT + 0.011555 * S + -0.0001152 * (S * S)) + pK1);
    c.K2 = exp(LN10 * (-25.9290 + -471.78 * iT + 0.01781 * S + -0.0001122 * (S * S) + 3.16967 * lT) + pK2);
    // KB: Dickson (1990) (:202-250)
    c.KB = exp(148.0248 + (-8966.90 + -2890.53 * sS + -77.942 * S + 1.728 * S * sS + -0.0996 * (S * S)) * iT +
               137.1942 * sS + 1.62142 * S + (-24.4344 + -25.085 * sS + -0.2474 * S) * lT + 0.053105 * sS * Tk + pKB);
    // KW: Millero (1995) (:279-313)
    c.KW = exp(148.9652 + -13847.26 * iT + -23.6521 * lT + (-5.977 + 118.67 * iT + 1.0495 * lT) * sS + -0.01615 * S + pKW);
    // KS: Dickson (1990) (:366-419); log(1 - 0.001005 S) is shared with KSi
    const double lS = log(1 + -0.001005 * S);
    c.KS = exp(141.328 + -4276.1 * iT + -23.093 * lT + (324.57 + -13856.0 * iT + -47.986 * lT) * sIs +
               (-771.54 + 35474.0 * iT + 114.723 * lT) * Is + -2698.0 * Is * sIs * iT + 1776.0 * (Is * Is) * iT + lS + pKS);
    // KF: Perez & Fraga (1987) (:451-487); log_S and log_S_KS terms are zero by default
    c.KF = exp(-9.68 + 874.0 * iT + 0.111 * sS + pKF);
    // KP1..3: Millero (1995) (:511-651)
    c.KP1 = c.KP2 = c.KP3 = c.KSi = c.K0 = 0.0;
    if (c.phosphate != 0.0) {
    c.KP1 = exp(115.525 + -4576.752 * iT + -18.453 * lT + (0.69171 + -106.736 * iT) * sS + (-0.01844 + -0.65643 * iT) * S + pP1);
    c.KP2 = exp(172.0883 + -8814.715 * iT + -27.927 * lT + (1.3566 + -160.340 * iT) * sS + (-0.05778 + 0.37335 * iT) * S + pP2);
    c.KP3 = exp(-18.141 + -3070.75 * iT + (2.81197 + 17.27039 * iT) * sS + (-0.09984 + -44.99486 * iT) * S + pP3);
    }
    // KSi: Millero (1995) (:674-713), no pressure correction
    if (c.silicate != 0.0)
    c.KSi = exp(117.385 + -8904.2 * iT + -19.334 * lT + (3.5913 + -458.79 * iT) * sIs + (-1.5998 + 188.74 * iT) * Is +
                (0.07871 + -12.1652 * iT) * (Is * Is) + lS);
    // K0: Weiss (1974) (:65-80)
    if (need_K0) c.K0 = weiss_k0(Tk, S, lT, iT);
}

// Alkalinity residual and its derivative in H (alkalinity_residual.jl:18-75).  The seven
// denominators (H, the carbonate and phosphate polynomials, KB + H, KSi + H, H + KS(1 + ST/KS),
// H + KF) are inverted with one division: prefix products, one reciprocal of the full product,
// and a backward sweep (the product stays above 1e-120 for H in [1e-14, 1]).
__host__ __device__ inline void alk_residual(double H, const CarbConsts& p, double& f, double& df) {
    const double H2 = H * H, H3 = H2 * H;
    const double a0 = H;
    const double a1 = H2 + p.K1 * H + p.K1K2;                       // carbonate denominator
    const double a2 = H3 + p.KP1 * H2 + p.KP12 * H + p.KP123;       // phosphate denominator
    const double a3 = p.KB + H, a4 = p.KSi + H, a5 = H + p.KSsd, a6 = H + p.KF;
    const double q1 = a0 * a1, q2 = q1 * a2, q3 = q2 * a3, q4 = q3 * a4, q5 = q4 * a5, q6 = q5 * a6;
    double r = 1.0 / q6;
    const double r6 = r * q5; r *= a6;
    const double r5 = r * q4; r *= a5;
    const double r4 = r * q3; r *= a4;
    const double r3 = r * q2; r *= a3;
    const double ipd = r * q1; r *= a2;
    const double icd = r * a0;
    const double iH = r * a1;
    const double iqb = p.KB * r3, iqsi = p.KSi * r4, iqh = H * r5, iqf = H * r6;
    const double PKK = p.PKK;
    f = p.K1 * H * p.DIC * icd + 2 * p.DIC * p.K1K2 * icd + p.boron * iqb + p.KW * iH + PKK * H * ipd +
        2 * PKK * p.KP3 * ipd + p.silicate * iqsi - H * p.isd - p.sulfate * iqh - p.fluoride * iqf -
        p.phosphate * H3 * ipd - p.Alk;
    const double dcd = 2 * H + p.K1;
    const double dpd = 3 * H2 + 2 * p.KP1 * H + p.KP12;
    df = p.K1 * p.DIC * (p.K1K2 - H2) * icd * icd - dcd * 2 * p.DIC * p.K1K2 * icd * icd -
         p.boron * iqb * iqb * p.iKB - p.KW * (iH * iH) + PKK * ipd - dpd * PKK * H * ipd * ipd -
         dpd * 2 * PKK * p.KP3 * ipd * ipd - p.silicate * iqsi * iqsi * p.iKSi - p.isd -
         p.sulfate * p.KSsd * (r5 * r5) - p.fluoride * p.KF * (r6 * r6) -
         3 * p.phosphate * H2 * ipd - dpd * p.phosphate * H3 * ipd * ipd;
}

struct CarbSolve {
    double H;
    int iters;
    bool converged;
};

__host__ __device__ inline CarbSolve solve_H(const obgc_carbon_options& o, double H0, const CarbConsts& p) {
    double x = H0, f, df;
    alk_residual(x, p, f, df);
    int N = 0;
    bool stalled = false, quadratic = false;
    const double lm = o.min_damping, c = o.armijo_constant;
    while (fabs(f) > o.atol && N < o.max_iters && !stalled) {
        const double d = f / df;
        double lam = 1.0;
        {   // bounded_lambda with lower bound 0 (solvers.jl:222-227)
            const double lb = x / d;
            lam = lb < 0 ? 1.0 : (lb < 1.0 ? lb : (lb == lb ? 1.0 : lb));
        }
        // A full step below 1e-9 of H is inside Newton's quadratic region: the iterate it reaches
        // is exact to FP64 resolution (the next step would be ~1e-18 of H), and the residual there
        // is rounding noise, where the Armijo test fails at random and backtracking to the minimum
        // damping only shortens the step.  Take it and stop, without evaluating the residual again.
        if (lam == 1.0 && fabs(d) <= 1e-9 * fabs(x)) {
            x -= d;
            N += 1;
            quadratic = true;
            break;
        }
        double fn, dfn;
        alk_residual(x - lam * d, p, fn, dfn);
        const double sf = f > 0 ? 1.0 : (f < 0 ? -1.0 : 0.0);
        while (fabs(fn) >= fabs(f) - c * lam * f * sf && lam > lm) {
            lam *= o.damping;
            alk_residual(x - lam * d, p, fn, dfn);
        }
        const double xn = x - lam * d;
        stalled = fabs(xn - x) <= 4e-16 * fabs(x);
        x = xn;
        f = fn;
        df = dfn;
        N += 1;
    }
    CarbSolve r;
    r.H = x;
    r.iters = N;
    // converged: residual below atol, or the iterate stopped moving at a residual that is rounding
    // noise relative to the alkalinity scale
    r.converged = quadratic || fabs(f) <= o.atol || (stalled && fabs(f) <= 1e-12 * (fabs(p.Alk) + fabs(p.DIC)) + 1e-30);
    if (!r.converged || !(x > 0)) {
        // bisection guard on the residual, decreasing in H over [1e-14, 1]
        double lo = 1e-14, hi = 1.0, flo, fhi, dd;
        alk_residual(lo, p, flo, dd);
        alk_residual(hi, p, fhi, dd);
        if (flo > 0 && fhi < 0) {
            for (int q = 0; q < 200; q++) {
                const double mid = sqrt(lo * hi);
                double fm;
                alk_residual(mid, p, fm, dd);
                if (fm > 0) lo = mid; else hi = mid;
                if (hi - lo <= 2e-16 * hi) break;
            }
            r.H = 0.5 * (lo + hi);
            r.converged = true;
        }
    }
    return r;
}

// pCO2 from fCO2 (carbon_chemistry.jl:170-193): the virial fugacity coefficient iterated three
// times at total pressure Pp (Pa).
__host__ __device__ inline double pco2_from_fco2(double fCO2, double Tk, double Pp) {
    const double B = (-1636.75 + 12.0408 * Tk + (-3.27957 * 1e-2) * (Tk * Tk) + (3.16528 * 1e-5) * (Tk * Tk * Tk)) * 1e-6;
    const double dl = (57.7 + -0.118 * Tk) * 1e-6;
    const double fp = fCO2 * 0.09807;
    double phi = 1.0, x = fp / Pp;
    for (int n = 0; n < 3; n++) {
        const double y = 1.0 - x;
        phi = exp((B + 2.0 * y * y * dl) * Pp / (8.31446261815324 * Tk));
        x = fp / (phi * Pp);
    }
    return fp / phi / 0.09807;
}

// One cell of (p::CarbonChemistry)(; DIC, T, S, Alk, pH, P, output, silicate, phosphate) and of
// carbonate_concentration / calcite_saturation.  Returns the selected output.
__host__ __device__ inline double carbon_cell(const obgc_carbon_options& o, double DIC, double Alk, double T, double S,
                                              double silicate, double phosphate, double P, double pH, double H_start,
                                              double* H_out, int* iters, bool* converged) {
    const bool carbonate_path = o.output == OBGC_OUT_CARBONATE || o.output == OBGC_OUT_OMEGA_CALCITE;
    const bool hasP = o.has_pressure != 0;
    const double Pd = hasP ? P : (carbonate_path ? 0.0 : 1.0);
    const double rho = seawater_density(o, T, S, Pd);
    CarbConsts c;
    c.boron = 0.000232 / 10.811 * S / 1.80655;
    c.sulfate = 0.14 / 96.06 * S / 1.80655;
    c.fluoride = 0.000067 / 18.9984 * S / 1.80655;
    const double Tk = T + 273.15;
    const double conv = 1e-3 / rho;
    c.Alk = Alk * conv;
    c.DIC = DIC * conv;
    c.phosphate = phosphate * conv;
    c.silicate = silicate * conv;
    equilibrium_constants(Tk, S, hasP, P, o.output == OBGC_OUT_FCO2 || o.output == OBGC_OUT_PCO2, c);
    prepare_residual(c);
    double H;
    int it = 0;
    bool ok = true;
    if (o.ph_given) {
        H = exp(-2.302585092994046 * pH);
    } else {
        const CarbSolve r = solve_H(o, H_start, c);
        H = r.H;
        it = r.iters;
        ok = r.converged;
    }
    if (H_out) *H_out = H;
    if (iters) *iters = it;
    if (converged) *converged = ok;
    if (carbonate_path) {
        const double d1 = H * (H + c.K1);
        const double d2 = 1.0 + c.K1 * c.K2 / d1;
        const double co3 = c.DIC * c.K1 * c.K2 / d1 / d2;
        if (o.output == OBGC_OUT_CARBONATE) return co3;
        // KSP_calcite / KSP_aragonite (equilibrium_constants.jl:740-850; log10(T) as in the reference)
        const bool arag = o.saturation_mineral == 1;
        const double pc = hasP ? pressure_log(arag ? -45.96 : -48.76, 0.5304, -0.0, -0.01176, 0.0003692, Tk, P, c.iRT) : 0.0;
        const double lnK = arag ? -171.945 + -0.077993 * Tk + 2903.293 * c.iT + 71.595 * (c.lT * 0.4342944819032518) +
                                      (-0.068393 + 0.0017276 * Tk + 88.135 * c.iT) * c.sS + -0.10018 * S + 0.0059415 * S * c.sS
                                : -171.9065 + -0.077993 * Tk + 2839.319 * c.iT + 71.595 * (c.lT * 0.4342944819032518) +
                                      (-0.77712 + 0.0028426 * Tk + 178.34 * c.iT) * c.sS + -0.07711 * S + 0.0041249 * S * c.sS;
        const double KSP = exp(2.302585092994046 * lnK + pc);
        return o.calcium_ion_per_salinity * S * co3 / KSP;
    }
    const double CO2 = c.DIC * (H * H) / (H * H + c.K1 * H + c.K1 * c.K2);
    const double fCO2 = (CO2 / c.K0) * 1e6;
    switch (o.output) {
        case OBGC_OUT_FCO2: return fCO2;
        case OBGC_OUT_H: return H;
        case OBGC_OUT_PH_FREE: return -log10(H);
        case OBGC_OUT_PCO2: return pco2_from_fco2(fCO2, Tk, (hasP ? P : 1.0) * 101325);
        case OBGC_OUT_PH_TOTAL: return -log10(H + c.sulfate / (1 + c.KS / H));
        case OBGC_OUT_PH_SWS: return -log10(H + c.sulfate / (1 + c.KS / H) + c.fluoride / (1 + c.KF / H));
    }
    return 0.0;
}

}  // namespace obgc
