// multig_device.cuh — SimpleMultiGSediment, nitrogen-only form (src/Models/Sediments/
// simple_multi_G.jl:15-430, sinking_carbon = nothing): the sediment fields' tendencies, its RK3 step
// and the tendencies it couples into the bottom cells of NO3, NH4 and O2.  FP64 in every precision:
// one thread per column does this once per RK3 stage of the water.
#pragma once
#include <math.h>
#include "../../include/obgc.h"

namespace obgc {

constexpr double MG_DAY = 86400.0;

// The parameters in the form the functors use them.
struct MultiG {
    double lf, ls;          // fast / slow decay rates (1/s)
    double ff, fs, fr;      // fast, slow, refractory fractions
    double R;               // sinking_redfield (C:N)
    double kO2;             // anoxia half saturation
    double ps;              // solid deposition fraction 0.223 sedimentation_rate^0.336
    double nox[6], den[6], anx[6];
};

inline MultiG make_multig(const obgc_multig_params& p) {
    MultiG m;
    m.lf = p.fast_decay_rate; m.ls = p.slow_decay_rate;
    m.ff = p.fast_fraction; m.fs = p.slow_fraction; m.fr = p.refactory_fraction;
    m.R = p.sinking_redfield;
    m.kO2 = p.anoxia_half_saturation;
    // simple_multi_G.jl:426: the constants 0.223 and 0.336 are written into the function (the
    // solid_dep_params tuple is not read)
    m.ps = 0.223 * pow(p.sedimentation_rate, 0.336);
    for (int q = 0; q < 6; q++) { m.nox[q] = p.nitrate_oxidation[q]; m.den[q] = p.denitrification[q]; m.anx[q] = p.anoxic[q]; }
    return m;
}

// Tendencies of (Ns, Nf, Nr) from the deposited nitrogen flux (simple_multi_G.jl:163-189).
__host__ __device__ inline void multig_fields_tendency(const MultiG& m, double Ns, double Nf, double flux, double G[3]) {
    G[0] = (1 - m.fr) * m.fs * flux - m.ls * Ns;
    G[1] = (1 - m.fr) * m.ff * flux - m.lf * Nf;
    G[2] = m.fr * flux;
}

// A fraction p of the Soetaert et al. (2000) fits, zero where it is not finite (simple_multi_G.jl:379,
// 395, 410: ifelse(isfinite(p), p, 0); a log of a negative or zero concentration gives NaN or -Inf).
__host__ __device__ inline double mg_finite_or_zero(double p) { return isfinite(p) ? p : 0.0; }

// The tendencies the sediment couples into the water's bottom cell (mmol/m2/s; simple_multi_G.jl:193-247
// and the fractions :352-424).  Nrm: the remineralisation rate ls Ns + lf Nf; Cr = Nrm R.
__host__ __device__ inline void multig_coupling(const MultiG& m, double Ns, double Nf, double NO3, double NH4, double O2,
                                                double* F_NO3, double* F_NH4, double* F_O2) {
    const double Nrm = m.ls * Ns + m.lf * Nf;
    const double Cr = Nrm * m.R;
    // reactivity(s, Ns R, Nf R) = (ls Cs + lf Cf) / (Cs + Cf + eps(0.0))
    const double Cs = Ns * m.R, Cf = Nf * m.R;
    const double k = (m.ls * Cs + m.lf * Cf) / (Cs + Cf + 4.9406564584124654e-324);
    const double lCr = log(Cr * MG_DAY), lk = log(k * MG_DAY), lkr = log(k);
    const double lO2 = log(O2), lNH4 = log(NH4), lNO3 = log(NO3);
    const double oxic = O2 / (m.kO2 + O2);
    const double* a = m.nox;
    const double pn = mg_finite_or_zero(exp(a[0] + a[1] * lCr * lO2 + a[2] * lCr * lCr + a[3] * lk * lNH4 + a[4] * lCr +
                                            a[5] * lCr * lNH4) / (Nrm * MG_DAY) * oxic);
    const double* b = m.den;
    const double pd = mg_finite_or_zero(exp(b[0] + b[1] * lCr + b[2] * lNO3 * lNO3 + b[3] * lCr * lCr + b[4] * lk * lk +
                                            b[5] * lO2 * lkr) / (Cr * MG_DAY) * oxic);
    const double* c = m.anx;
    const double pa = mg_finite_or_zero(exp(c[0] + c[1] * lCr + c[2] * lCr * lCr + c[3] * lk + c[4] * lO2 * lkr +
                                            c[5] * lNO3 * lNO3) / (Cr * MG_DAY));
    *F_NH4 = (1 - pn) * Nrm + 0.8 * pd * Cr;
    *F_NO3 = pn * Nrm - 0.8 * pd * Cr;
    *F_O2 = -(1 - pa * m.ps - pd) * oxic * Cr - 2 * pn * Nrm;
}

}  // namespace obgc
