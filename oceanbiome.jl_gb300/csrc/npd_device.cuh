// npd_device.cuh — the NutrientsPlanktonDetritus tracer functors, evaluated for ALL tracers of a
// cell at once.  The reference evaluates one functor per tracer per cell, each recomputing the
// shared sub-terms (phytoplankton_growth in ≥7 functors, total_grazing in ≥5, and Alk/O₂ calling
// whole NH₄/NO₃ functors); here each sub-term is computed once and every tendency is assembled
// from them, in the reference's arithmetic order.  Formulas follow
// src/Models/AdvectedPopulations/NutrientsPlanktonDetritus/{nutrients,plankton,detritus,
// carbonate_system,oxygen}.jl (line references at each term).
//
// Template parameter V selects compile-time component kinds for the fused 3-D kernels
// (V >= 0, table below); V = -1 reads every kind from the parameter struct at run time.
#pragma once
#include "obgc_common.cuh"

namespace obgc {

template <typename T>
struct NPDParamsT {
    int nutrients, detritus, carbonate_system, oxygen, light_limitation, q10, pmort, graz;
    T nitrification_rate;
    T kNO3, kNH4, kFe, psi, kPAR, mu0, R_Fe, gamma, alpha_exud, Q10, mP, mZ, mu_ex, alpha_solid,
      alpha_exinorg, p_pref, g_max, kG, alpha_assim, calc_diss_zoo, R, rho_calc, eta_gut, R_chl;
    T rem_inorg, s_rem, l_rem, d_rem, f_small, R_det;
    T D_rem, f_small_D;
    T Rp, Rn;
};

template <typename T>
__host__ __device__ inline NPDParamsT<T> make_params(const obgc_npd_params& p) {
    NPDParamsT<T> o;
    o.nutrients = p.nutrients; o.detritus = p.detritus; o.carbonate_system = p.carbonate_system;
    o.oxygen = p.oxygen; o.light_limitation = p.light_limitation;
    o.q10 = p.has_temperature_coefficient; o.pmort = p.phytoplankton_mortality_formulation;
    o.graz = p.grazing_concentration_formulation;
    o.nitrification_rate = T(p.nitrification_rate);
    o.kNO3 = T(p.nitrate_half_saturation); o.kNH4 = T(p.ammonia_half_saturation);
    o.kFe = T(p.iron_half_saturation); o.psi = T(p.nitrate_ammonia_inhibition);
    o.kPAR = T(p.light_half_saturation); o.mu0 = T(p.phytoplankton_maximum_growth_rate);
    o.R_Fe = T(p.iron_ratio); o.gamma = T(p.phytoplankton_exudation_fraction);
    o.alpha_exud = T(p.ammonia_fraction_of_exudate); o.Q10 = T(p.temperature_coefficient);
    o.mP = T(p.phytoplankton_mortality_rate); o.mZ = T(p.zooplankton_mortality_rate);
    o.mu_ex = T(p.zooplankton_excretion_rate); o.alpha_solid = T(p.phytoplankton_solid_waste_fraction);
    o.alpha_exinorg = T(p.excretion_inorganic_fraction); o.p_pref = T(p.preference_for_phytoplankton);
    o.g_max = T(p.maximum_grazing_rate); o.kG = T(p.grazing_half_saturation);
    o.alpha_assim = T(p.zooplankton_assimilation_fraction);
    o.calc_diss_zoo = T(p.zooplankton_calcite_dissolution); o.R = T(p.redfield_ratio);
    o.rho_calc = T(p.carbon_calcite_ratio); o.eta_gut = T(p.zooplankton_gut_calcite_dissolution);
    o.R_chl = T(p.phytoplankton_chlorophyll_ratio);
    o.rem_inorg = T(p.remineralisation_inorganic_fraction); o.s_rem = T(p.small_remineralisation_rate);
    o.l_rem = T(p.large_remineralisation_rate); o.d_rem = T(p.dissolved_remineralisation_rate);
    o.f_small = T(p.small_solid_waste_fraction); o.R_det = T(p.detritus_redfield_ratio);
    o.D_rem = T(p.detritus_remineralisation_rate); o.f_small_D = T(p.small_particle_fraction);
    o.Rp = T(p.respiration_oxygen_nitrogen_ratio); o.Rn = T(p.nitrification_oxygen_nitrogen_ratio);
    return o;
}

// Named values of one cell (tracers by enum obgc_tracer order).
template <typename T>
struct NPDVals {
    T v[OBGC_NUM_NAMED];
};

// Compile-time variants of the fused kernels: {nutrients, detritus, carbonate, oxygen, q10}.
// V_EXTERNAL: the fused substep takes its BGC tendencies from arrays computed by another kernel
// (PISCES), keeping the advection, sinking and RK3 update.
enum Variant { V_RUNTIME = -1, V_LOBSTER = 0, V_LOBSTER_C = 1, V_LOBSTER_CO = 2, V_NPZD = 3, V_LOBSTER_O = 4, V_EXTERNAL = 5 };
__host__ __device__ constexpr int vnut(int V) { return V == V_NPZD ? OBGC_NUT_NUTRIENT : OBGC_NUT_NITRATE_AMMONIA; }
__host__ __device__ constexpr int vdet(int V) { return V == V_NPZD ? OBGC_DET_SINGLE : OBGC_DET_TWO_PARTICLE; }
__host__ __device__ constexpr int vcarb(int V) { return (V == V_LOBSTER_C || V == V_LOBSTER_CO) ? 1 : 0; }
__host__ __device__ constexpr int voxy(int V) { return (V == V_LOBSTER_CO || V == V_LOBSTER_O) ? 1 : 0; }
__host__ __device__ constexpr int vq10(int V) { return V == V_NPZD ? 1 : 0; }

// Which variant (if any) a parameter set corresponds to; -1 if none.
inline int variant_of(const obgc_npd_params& p) {
    for (int V = 0; V <= 4; V++) {
        if (p.nutrients == vnut(V) && p.detritus == vdet(V) && p.carbonate_system == vcarb(V) &&
            p.oxygen == voxy(V) && p.has_temperature_coefficient == vq10(V))
            return V;
    }
    return -1;
}

// Fused evaluation of every tendency of the model at one point.  G receives the tendencies of
// the model's tracers (others untouched).
// Division by a denominator bounded away from zero (a half-saturation constant plus a
// concentration): the fast FP32 division on the device (<= 2 ulp), IEEE division otherwise.
template <typename T>
__host__ __device__ __forceinline__ T qdiv(T a, T b) {
#ifdef __CUDA_ARCH__
    if constexpr (sizeof(T) == 4) return __fdividef(a, b);
#endif
    return a / b;
}

// Lt_given: the temperature factor Q10^(T/10) already evaluated for this v[OBGC_T] (a caller whose
// temperature does not change between calls, such as a box model, saves the pow), or NULL.
template <int V, typename T>
__host__ __device__ inline void npd_tendencies(const NPDParamsT<T>& p, const T* v, T PAR, T* G, const T* Lt_given = nullptr) {
    const int nut = V >= 0 ? vnut(V) : p.nutrients;
    const int det = V >= 0 ? vdet(V) : p.detritus;
    const int carb = V >= 0 ? vcarb(V) : p.carbonate_system;
    const int oxy = V >= 0 ? voxy(V) : p.oxygen;
    const int q10 = V >= 0 ? vq10(V) : p.q10;
    const T one = T(1), two = T(2);
    const T P = v[OBGC_P], Z = v[OBGC_Z];

    // small / large particulate and dissolved concentrations (detritus.jl:41-57,103-119,295-308)
    T sP, lP = 0, dN = 0, sPC = 0, lPC = 0, dC = 0;
    if (det == OBGC_DET_TWO_PARTICLE) {
        sP = v[OBGC_SPOM]; lP = v[OBGC_BPOM]; dN = v[OBGC_DOM];
        sPC = v[OBGC_SPOM] * p.R_det; lPC = v[OBGC_BPOM] * p.R_det; dC = v[OBGC_DOM] * p.R_det;
    } else if (det == OBGC_DET_VARIABLE_REDFIELD) {
        sP = v[OBGC_SPON]; lP = v[OBGC_BPON]; dN = v[OBGC_DON];
        sPC = v[OBGC_SPOC]; lPC = v[OBGC_BPOC]; dC = v[OBGC_DOC];
    } else if (det == OBGC_DET_SINGLE) {
        sP = v[OBGC_D] * p.f_small_D;
    } else {
        sP = T(0);
    }

    // grazing (plankton.jl:118-135, 352-397)
    const T pp = p.p_pref * P / (p.p_pref * P + (one - p.p_pref) * sP + tiny<T>());
    const T food = pp * P + (one - pp) * sP;
    const T L = p.graz == OBGC_LINEAR ? qdiv(food, food + p.kG) : qdiv(food * food, food * food + p.kG * p.kG);
    const T Gtot = p.g_max * L * Z;
    const T fden = food + jl_eps(food);
    // the eps-guarded denominators need true division: their reciprocal overflows at zero
    const T GP = p.g_max * pp * L * P / fden * Z;
    const T Gs = p.g_max * (one - pp) * L * sP / fden * Z;
    const T nuP = p.pmort == OBGC_LINEAR ? p.mP * P : p.mP * (P * P);

    // growth (plankton.jl:150-220)
    T nl = 0, al = 0, Ln;
    if (nut != OBGC_NUT_NUTRIENT) {
        const T NO3 = v[OBGC_NO3], NH4 = v[OBGC_NH4];
        nl = qdiv(NO3 * t_exp(-p.psi * NH4), NO3 + p.kNO3);
        al = t_max0(qdiv(NH4, p.kNH4 + NH4));
        Ln = (nl + al) / two;
        if (nut == OBGC_NUT_NITRATE_AMMONIA_IRON) Ln = Ln * (v[OBGC_FE] / (p.kFe + v[OBGC_FE]));
    } else {
        Ln = qdiv(v[OBGC_N], v[OBGC_N] + p.kNO3);
    }
    const T Ll = p.light_limitation == OBGC_LIGHT_MONDO ? qdiv(PAR, p.kPAR + PAR)
                                                          : PAR / t_sqrt(PAR * PAR + p.kPAR * p.kPAR);
    const T Lt = q10 ? (Lt_given ? *Lt_given : t_pow(p.Q10, v[OBGC_T] / T(10))) : one;
    const T muP = p.mu0 * Ll * Ln * Lt * P;

    // wastes (plankton.jl:292-349)
    const T pinw = p.alpha_exinorg * p.mu_ex * Z + (one - p.alpha_solid) * nuP;
    const T ponw = (one - p.alpha_exud) * p.gamma * muP + (one - p.alpha_exinorg) * p.mu_ex * Z;
    const T sw = (one - p.alpha_assim) * Gtot + p.alpha_solid * nuP + p.mZ * (Z * Z);

    // detritus wastes (detritus.jl:161-207, 298-317)
    T dinw, donw = 0, dicw, docw = 0;
    if (det == OBGC_DET_TWO_PARTICLE || det == OBGC_DET_VARIABLE_REDFIELD) {
        dinw = p.rem_inorg * (p.s_rem * sP + p.l_rem * lP) + p.d_rem * dN;
        donw = (one - p.rem_inorg) * (p.s_rem * sP + p.l_rem * lP);
        dicw = p.rem_inorg * (p.s_rem * sPC + p.l_rem * lPC) + p.d_rem * dC;
        docw = (one - p.rem_inorg) * (p.s_rem * sPC + p.l_rem * lPC);
    } else if (det == OBGC_DET_SINGLE) {
        dinw = v[OBGC_D] * p.D_rem;
        dicw = v[OBGC_D] * p.D_rem * p.R_det;
    } else {
        dinw = ponw + sw;
        dicw = (ponw + sw) * p.R;
    }

    // nutrients (nutrients.jl:154-191; uptake plankton.jl:223-278)
    T tNH4 = 0, tNO3 = 0, tN = 0, nitrif = 0;
    if (nut != OBGC_NUT_NUTRIENT) {
        nitrif = p.nitrification_rate * v[OBGC_NH4];
        const T upNO3 = muP * nl / (nl + al + tiny<T>());
        const T upNH4 = muP * al / (nl + al + tiny<T>()) - p.alpha_exud * p.gamma * muP;
        tNO3 = nitrif - upNO3;
        tNH4 = pinw + dinw - nitrif - upNH4;
        G[OBGC_NO3] = tNO3;
        G[OBGC_NH4] = tNH4;
        if (nut == OBGC_NUT_NITRATE_AMMONIA_IRON) G[OBGC_FE] = -(p.R_Fe * muP);
    } else {
        tN = pinw + dinw - muP * (one - p.alpha_exud * p.gamma);
        G[OBGC_N] = tN;
    }

    // plankton (plankton.jl:92-116)
    G[OBGC_P] = (one - p.gamma) * muP - GP - nuP;
    G[OBGC_Z] = p.alpha_assim * Gtot - p.mZ * (Z * Z) - p.mu_ex * Z;

    // detritus (detritus.jl:85-101, 143-158, 282-288)
    if (det == OBGC_DET_TWO_PARTICLE) {
        G[OBGC_DOM] = ponw + donw - p.d_rem * dN;
        G[OBGC_SPOM] = p.f_small * sw - Gs - p.s_rem * sP;
        G[OBGC_BPOM] = (one - p.f_small) * sw - p.l_rem * lP;
    } else if (det == OBGC_DET_VARIABLE_REDFIELD) {
        G[OBGC_DON] = ponw + donw - p.d_rem * dN;
        G[OBGC_SPON] = p.f_small * sw - Gs - p.s_rem * sP;
        G[OBGC_BPON] = (one - p.f_small) * sw - p.l_rem * lP;
        const T calc_prod = (GP * (one - p.eta_gut) + nuP) * p.rho_calc * p.R;
        G[OBGC_SPOC] = p.f_small * (sw * p.R) - Gs * p.R - p.s_rem * sPC;
        G[OBGC_BPOC] = (one - p.f_small) * (sw * p.R) + calc_prod - p.l_rem * lPC;
        G[OBGC_DOC] = p.R * ponw + docw - p.d_rem * dC;
    } else if (det == OBGC_DET_SINGLE) {
        G[OBGC_D] = ponw + sw - Gs - p.D_rem * v[OBGC_D];
    }

    // carbonate system (carbonate_system.jl:49-67; calcite terms plankton.jl:399-450)
    if (carb) {
        const T calc_diss = det == OBGC_DET_VARIABLE_REDFIELD ? GP * p.eta_gut * p.rho_calc * p.R
                                                               : (GP + nuP) * p.rho_calc * p.R;
        const T calc_up = two * p.rho_calc * muP * p.R;
        const T PPd = (one + p.rho_calc * (one - p.gamma) - p.alpha_exud * p.gamma) * muP * p.R;
        G[OBGC_DIC] = -PPd + p.R * pinw + dicw + calc_diss;
        if (nut != OBGC_NUT_NUTRIENT)
            G[OBGC_ALK] = tNH4 * T(1 - 1.0 / 16) - tNO3 * T(1 + 1.0 / 16) - two * calc_up + two * calc_diss;
        else
            G[OBGC_ALK] = tN - two * calc_up + two * calc_diss;
    }
    // oxygen (oxygen.jl:21-31; the NH₄ functor is the zero fallback for Nutrient)
    if (oxy) G[OBGC_O2] = p.Rp * muP - (p.Rp - p.Rn) * tNH4 - p.Rp * nitrif;
}

}  // namespace obgc
