// pisces_device.cuh — every PISCES tendency of one cell, computed in one pass.
//
// The reference evaluates each of the 24 tracers with its own functor, and each functor recomputes
// the nutrient limitations, growth rates, grazing and bacterial terms it needs (the nutrient
// limitation alone is evaluated dozens of times per cell).  Here every shared term is evaluated
// once and all 24 tendencies are assembled from them, in the reference's arithmetic
// (src/Models/AdvectedPopulations/PISCES/, functions named alongside).  Kept as the reference has
// them: the growth rate's day length with latitude and time swapped (growth_rate.jl:29; the host
// evaluates both day lengths once per call), negative sinking velocities in the flux feeding,
// nitrogen fixation's comparison of a rate in 1/s with 2.15, the bacteria cap of 4.
#pragma once
#include "obgc_common.cuh"

namespace obgc {

template <typename T>
struct PhytoT {
    int growth_kind, silicate_limited;
    T delta, b1, b2, b3, Km, m_lin, w0, w1, th0_chl, th1_chl, th_fe_max, K1_si, K2_si, th0_si, k_fe, I_m, S_size;
    T mu0, b_T, dark_tol, alpha0, beta, b_r, mu_r;
    T k_nh4, k_no3, k_po4, th_opt_fe, k_si, pk_si;
};

template <typename T>
struct ZooT {
    T b_T, g0, pP, pD, pPOC, pZ, thr, J, K, gf0, th_fe, e0, sigma, Km, m0, r, gamma, eta;
};

template <typename T>
struct PiscesT {
    PhytoT<T> ph[2];                 // nano, diatoms
    T rain0;
    ZooT<T> zo[2];                   // micro, meso
    T bZ, bM, bdepth, K_doc_b, K_no3_b, K_nh4_b, K_po4_b, K_fe_b;
    T lam_doc, bact_ref, b_doc, a_doc[5];
    T b_pom, lam_pom, a_pom[4], lam_fe0, lam_fe1, kappa_bact, kappa_small, kappa_large, chi0, lam_fast, lam_slow;
    T lam_ca, n_ca, th_bact_fe, K_bact_fe, mu_bact;
    T lam_nitrif, N_fix, K_fe_fix, K_po4_fix, E_fix;
    T scav_enh, L_max, L_ratio;
    T th_resp, th_nitrif;
    T min1, min2, thN, thP, shear_ml, shear_bg, latitude;
    T w_poc, w_goc_min, w_goc_max;
    int open_bottom;
};

template <typename T>
inline PhytoT<T> make_phyto(const obgc_pisces_phyto& c) {
    PhytoT<T> o;
    o.growth_kind = c.growth_kind; o.silicate_limited = c.silicate_limited;
    o.delta = T(c.exudated_fraction); o.b1 = T(c.blue_light_absorption); o.b2 = T(c.green_light_absorption);
    o.b3 = T(c.red_light_absorption); o.Km = T(c.mortality_half_saturation); o.m_lin = T(c.linear_mortality_rate);
    o.w0 = T(c.base_quadratic_mortality); o.w1 = T(c.maximum_quadratic_mortality);
    o.th0_chl = T(c.minimum_chlorophyll_ratio); o.th1_chl = T(c.maximum_chlorophyll_ratio);
    o.th_fe_max = T(c.maximum_iron_ratio); o.K1_si = T(c.silicate_half_saturation);
    o.K2_si = T(c.enhanced_silicate_half_saturation); o.th0_si = T(c.optimal_silicate_ratio);
    o.k_fe = T(c.half_saturation_for_iron_uptake); o.I_m = T(c.threshold_for_size_dependency); o.S_size = T(c.size_ratio);
    o.mu0 = T(c.base_growth_rate); o.b_T = T(c.temperature_sensitivity); o.dark_tol = T(c.dark_tolerance);
    o.alpha0 = T(c.initial_slope_of_PI_curve); o.beta = T(c.low_light_adaptation);
    o.b_r = T(c.basal_respiration_rate); o.mu_r = T(c.reference_growth_rate);
    o.k_nh4 = T(c.minimum_ammonium_half_saturation); o.k_no3 = T(c.minimum_nitrate_half_saturation);
    o.k_po4 = T(c.minimum_phosphate_half_saturation); o.th_opt_fe = T(c.optimal_iron_quota);
    o.k_si = T(c.minimum_silicate_half_saturation); o.pk_si = T(c.silicate_half_saturation_parameter);
    return o;
}

template <typename T>
inline ZooT<T> make_zoo(const obgc_pisces_zoo& z) {
    ZooT<T> o;
    o.b_T = T(z.temperature_sensitivity); o.g0 = T(z.maximum_grazing_rate);
    o.pP = T(z.preference_P); o.pD = T(z.preference_D); o.pPOC = T(z.preference_POC); o.pZ = T(z.preference_Z);
    o.thr = T(z.food_threshold_concentration); o.J = T(z.specific_food_threshold_concentration);
    o.K = T(z.grazing_half_saturation); o.gf0 = T(z.maximum_flux_feeding_rate); o.th_fe = T(z.iron_ratio);
    o.e0 = T(z.minimum_growth_efficiency); o.sigma = T(z.non_assimilated_fraction); o.Km = T(z.mortality_half_saturation);
    o.m0 = T(z.quadratic_mortality); o.r = T(z.linear_mortality); o.gamma = T(z.dissolved_excretion_fraction);
    o.eta = T(z.undissolved_calcite_fraction);
    return o;
}

template <typename T>
inline PiscesT<T> make_pisces(const obgc_pisces_params& p) {
    PiscesT<T> o;
    o.ph[0] = make_phyto<T>(p.nano); o.ph[1] = make_phyto<T>(p.diatoms);
    o.rain0 = T(p.base_rain_ratio);
    o.zo[0] = make_zoo<T>(p.micro); o.zo[1] = make_zoo<T>(p.meso);
    o.bZ = T(p.micro_bacteria); o.bM = T(p.meso_bacteria); o.bdepth = T(p.bacteria_depth_exponent);
    o.K_doc_b = T(p.doc_half_saturation_bacteria); o.K_no3_b = T(p.nitrate_half_saturation_bacteria);
    o.K_nh4_b = T(p.ammonia_half_saturation_bacteria); o.K_po4_b = T(p.phosphate_half_saturation_bacteria);
    o.K_fe_b = T(p.iron_half_saturation_bacteria);
    o.lam_doc = T(p.doc_remineralisation_rate); o.bact_ref = T(p.doc_reference_bacteria); o.b_doc = T(p.doc_temperature_sensitivity);
    for (int q = 0; q < 5; q++) o.a_doc[q] = T(p.doc_aggregation[q]);
    o.b_pom = T(p.pom_temperature_sensitivity); o.lam_pom = T(p.pom_base_breakdown_rate);
    for (int q = 0; q < 4; q++) o.a_pom[q] = T(p.pom_aggregation[q]);
    o.lam_fe0 = T(p.minimum_iron_scavenging_rate); o.lam_fe1 = T(p.load_specific_iron_scavenging_rate);
    o.kappa_bact = T(p.bacterial_iron_uptake_efficiency); o.kappa_small = T(p.small_fraction_bacterial_iron);
    o.kappa_large = T(p.large_fraction_bacterial_iron); o.chi0 = T(p.base_liable_silicate_fraction);
    o.lam_fast = T(p.fast_dissolution_rate_of_silicate); o.lam_slow = T(p.slow_dissolution_rate_of_silicate);
    o.lam_ca = T(p.base_calcite_dissolution_rate); o.n_ca = T(p.calcite_dissolution_exponent);
    o.th_bact_fe = T(p.maximum_iron_ratio_in_bacteria); o.K_bact_fe = T(p.iron_half_saturation_for_bacteria);
    o.mu_bact = T(p.maximum_bacterial_growth_rate);
    o.lam_nitrif = T(p.maximum_nitrification_rate); o.N_fix = T(p.maximum_fixation_rate);
    o.K_fe_fix = T(p.iron_half_saturation_for_fixation); o.K_po4_fix = T(p.phosphate_half_saturation_for_fixation);
    o.E_fix = T(p.light_saturation_for_fixation);
    o.scav_enh = T(p.excess_scavenging_enhancement); o.L_max = T(p.maximum_ligand_concentration);
    o.L_ratio = T(p.dissolved_ligand_ratio);
    o.th_resp = T(p.ratio_for_respiration); o.th_nitrif = T(p.ratio_for_nitrification);
    o.min1 = T(p.first_anoxia_threshold); o.min2 = T(p.second_anoxia_threshold);
    o.thN = T(p.nitrogen_redfield_ratio); o.thP = T(p.phosphate_redfield_ratio);
    o.shear_ml = T(p.mixed_layer_shear); o.shear_bg = T(p.background_shear); o.latitude = T(p.latitude);
    o.w_poc = T(p.poc_sinking_speed); o.w_goc_min = T(p.goc_minimum_speed); o.w_goc_max = T(p.goc_maximum_speed);
    o.open_bottom = p.open_bottom;
    return o;
}

// NaN-propagating min / max (Julia's min and max)
template <typename T>
__host__ __device__ __forceinline__ T jmin(T a, T b) { return (a != a || b != b) ? a + b : (a < b ? a : b); }
template <typename T>
__host__ __device__ __forceinline__ T jmax(T a, T b) { return (a != a || b != b) ? a + b : (a > b ? a : b); }

// Day lengths used by one evaluation: the growth rate's (latitude and time swapped, as the
// reference calls it) and the energy-assimilation ratio's (src/Utils/Utils.jl:18-34).
template <typename T>
struct PiscesClock {
    T day_length_growth, day_length_ratio;
};

template <typename T>
struct PiscesPhytoState {
    T I, IChl, IFe, L, LFe, LPO4, LN, LNO3, LNH4, mu_i, mu, muI, lin, quad, uFe;
};

template <typename T>
__host__ __device__ __forceinline__ T pis_pow(T a, T b) { return t_pow(a, b); }

// Nutrient limitation, growth, mortality and iron uptake of one class (phytoplankton/*.jl).
template <typename T>
__host__ __device__ inline PiscesPhytoState<T> pisces_phyto(const PhytoT<T>& ph, const PiscesT<T>& p, T I, T IChl, T IFe,
                                                         T NO3, T NH4, T PO4, T Si, T Fe, T Tc, const T* a, T z,
                                                         const PiscesClock<T>& clk) {
    const T e = tiny<T>();
    PiscesPhytoState<T> s;
    s.I = I; s.IChl = IChl; s.IFe = IFe;
    // size_factor (mixed_mondo.jl:207-215)
    const T I1 = jmin(I, ph.I_m), I2 = jmax(T(0), I - ph.I_m);
    const T Kb = (I1 + ph.S_size * I2) / (I1 + I2 + e);
    // NitrogenIronPhosphateSilicateLimitation (nutrient_limitation.jl:20-73)
    const T thFe = I == T(0) ? T(0) : IFe / (I + e);
    const T thChl = I == T(0) ? T(0) : IChl / (T(12) * I + e);
    const T Kno = ph.k_no3 * Kb, Knh = ph.k_nh4 * Kb, Kp = ph.k_po4 * Kb, Ksi = ph.k_si * Kb;
    s.LNO3 = (Knh * NO3) / (Kno * Knh + Kno * NH4 + Knh * NO3 + e);
    s.LNH4 = (Kno * NH4) / (Knh * Kno + Knh * NO3 + Kno * NH4 + e);
    s.LN = s.LNO3 + s.LNH4;
    s.LPO4 = PO4 / (PO4 + Kp + e);
    const T thm = T(1000) * (T(0.0016 / 55.85 * 12) * thChl + T(1.5 * 1.21e-5 * 14 / (55.85 * 7.625)) * s.LN +
                             T(1.15e-4 * 14 / (55.85 * 7.625)) * s.LNO3);
    s.LFe = jmin(T(1), jmax(T(0), (thFe - thm) / ph.th_opt_fe));
    const T Sic = a[OBGC_PAUX_SICLIM];
    const T KSi = Ksi + T(7) * Sic * Sic / (ph.pk_si * ph.pk_si + Sic * Sic);
    T L = jmin(jmin(s.LN, s.LPO4), s.LFe);
    if (ph.silicate_limited) L = jmin(L, Si / (Si + KSi));
    s.L = L;
    // BaseProduction (growth_rate.jl:3-45) with light_limitation (:77-83, :117-124)
    const T PAR = ph.b1 * a[OBGC_PAUX_PAR1] + ph.b2 * a[OBGC_PAUX_PAR2] + ph.b3 * a[OBGC_PAUX_PAR3];
    const T dzd = jmax(T(0), a[OBGC_PAUX_ZEU] - a[OBGC_PAUX_ZMXL]);
    const T drt = dzd * dzd / a[OBGC_PAUX_KAPPA];
    s.mu_i = ph.mu0 * pis_pow(ph.b_T, Tc);
    const T dl = clk.day_length_growth;
    const T f1 = T(1.5) * dl / (dl + T(0.5 * 86400.0));
    const T f2 = T(1) - drt / (drt + ph.dark_tol);
    const T alpha = ph.alpha0 * (T(1) + ph.beta * t_exp(-PAR));
    const T theta = IChl / (T(12) * I + e);
    const T fl = ph.growth_kind == 0 ? T(1) - t_exp(-alpha * theta * PAR / (dl * s.mu_i * L + e))
                                     : T(1) - t_exp(-alpha * theta * PAR / (dl * (ph.b_r + ph.mu_r)));
    s.mu = s.mu_i * f1 * f2 * fl * L;
    s.muI = s.mu * I;
    // mortality (mixed_mondo.jl:137-156)
    s.lin = ph.m_lin * I / (I + ph.Km) * I;
    const T w = ph.w0 + ph.w1 * T(0.25) * (T(1) - L * L) / (T(0.25) + L * L);
    const T shear = z < a[OBGC_PAUX_ZMXL] ? p.shear_bg : p.shear_ml;
    s.quad = shear * w * I * I;
    // iron_uptake (mixed_mondo.jl:177-197)
    const T Kfe = ph.k_fe * Kb;
    const T L1 = Fe / (Fe + Kfe + e);
    const T L2 = T(4) - T(4.5) * s.LFe / (s.LFe + T(1));
    const T r = IFe / (I + e) / ph.th_fe_max;
    s.uFe = (T(1) - ph.delta) * ph.th_fe_max * L1 * L2 * jmax(T(0), (T(1) - r) / (T(1.05) - r)) * s.mu_i * I;
    return s;
}

// All 24 tendencies of a cell.  v: 26 tracer values (PISCES order), a: 12 auxiliary values with
// the sinking velocities already interpolated to the cell centre; z: cell centre (m).
template <typename T>
__host__ __device__ inline void pisces_tendencies(const PiscesT<T>& p, const T* v, const T* a, T z,
                                                  const PiscesClock<T>& clk, T* G) {
    const T e = tiny<T>();
    const T P = v[OBGC_PIS_P], PChl = v[OBGC_PIS_PCHL], PFe = v[OBGC_PIS_PFE], D = v[OBGC_PIS_D], DChl = v[OBGC_PIS_DCHL];
    const T DFe = v[OBGC_PIS_DFE], DSi = v[OBGC_PIS_DSI], Z = v[OBGC_PIS_Z], M = v[OBGC_PIS_M], DOC = v[OBGC_PIS_DOC];
    const T POC = v[OBGC_PIS_POC], GOC = v[OBGC_PIS_GOC], SFe = v[OBGC_PIS_SFE], BFe = v[OBGC_PIS_BFE], PSi = v[OBGC_PIS_PSI];
    const T CaCO3 = v[OBGC_PIS_CACO3], NO3 = v[OBGC_PIS_NO3], NH4 = v[OBGC_PIS_NH4], PO4 = v[OBGC_PIS_PO4], Fe = v[OBGC_PIS_FE];
    const T Si = v[OBGC_PIS_SI], O2 = v[OBGC_PIS_O2], Tc = v[OBGC_PIS_T];
    const T zmxl = a[OBGC_PAUX_ZMXL], zeu = a[OBGC_PAUX_ZEU], wPOC = a[OBGC_PAUX_WPOC], wGOC = a[OBGC_PAUX_WGOC];
    const T shear = z < zmxl ? p.shear_bg : p.shear_ml;
    // anoxia_factor (common.jl:61-66)
    const T dO2 = jmin(T(1), jmax(T(0), T(0.4) * (p.min1 - O2) / (p.min2 + O2)));

    // ---- phytoplankton
    const PiscesPhytoState<T> n = pisces_phyto(p.ph[0], p, P, PChl, PFe, NO3, NH4, PO4, Si, Fe, Tc, a, z, clk);
    const PiscesPhytoState<T> d = pisces_phyto(p.ph[1], p, D, DChl, DFe, NO3, NH4, PO4, Si, Fe, Tc, a, z, clk);
    // production_and_energy_assimilation_absorption_ratio (growth_rate.jl:126-156)
    T rho[2];
    {
        const T dl = clk.day_length_ratio;
        const T f1 = T(1.5) * dl / (dl + T(0.5 * 86400.0));
        const PiscesPhytoState<T>* cl[2] = {&n, &d};
        for (int c = 0; c < 2; c++) {
            const PhytoT<T>& ph = p.ph[c];
            const T PAR = ph.b1 * a[OBGC_PAUX_PAR1] + ph.b2 * a[OBGC_PAUX_PAR2] + ph.b3 * a[OBGC_PAUX_PAR3];
            const T mu_check = cl[c]->mu / f1 * dl;
            const T alpha = ph.alpha0 * (T(1) + ph.beta * t_exp(-PAR));
            rho[c] = T(12) * mu_check * cl[c]->I / (alpha * cl[c]->IChl * PAR + e) * cl[c]->L;
        }
    }
    // uptake of NO3 and NH4 (mixed_mondo.jl:250-264)
    const T up_no3 = n.muI * n.LNO3 / (n.LN + e) + d.muI * d.LNO3 / (d.LN + e);
    const T up_nh4 = n.muI * n.LNH4 / (n.LN + e) + d.muI * d.LNH4 / (d.LN + e);
    const T production = n.muI + d.muI;
    // silicate_uptake (mixed_mondo.jl:217-248)
    T up_si;
    {
        const PhytoT<T>& ph = p.ph[1];
        const T L1 = Si / (Si + ph.K1_si + e);
        const T L2 = p.latitude < T(0) ? Si * Si * Si / (Si * Si * Si + ph.K2_si * ph.K2_si * ph.K2_si) : T(0);
        const T F1 = jmin(jmin(jmin(d.mu / (d.mu_i * d.L + e), d.LFe), d.LPO4), d.LN);
        const T F2 = jmin(T(1), T(2.2) * jmax(T(0), L1 - T(0.5)));
        const T th1 = ph.th0_si * L1 * jmin(T(5.4), (T(4.4) * t_exp(T(-4.23) * F1) * F2 + T(1)) * (T(1) + T(2) * L2));
        up_si = (T(1) - ph.delta) * th1 * d.mu * D;
    }

    // ---- zooplankton (food_quality_dependant.jl, grazing_waste.jl, iron_grazing.jl)
    const T food[4] = {P, D, POC, Z};
    const T iron_q[4] = {PFe / (P + e), DFe / (D + e), SFe / (POC + e), p.zo[0].th_fe};
    const T edible = POC * wPOC + GOC * wGOC;           // edible_flux_rate (two_size_class.jl:90-98)
    const T edible_fe = SFe * wPOC + BFe * wGOC;
    T gI[2], eff[2], gfI[2], gIFe[2], gfIFe[2], mort[2], spec[2], avail[2], gP[2], gD[2], gPOC[2], fPOC[2], fGOC[2];
    T gZ_meso = T(0);
    for (int c = 0; c < 2; c++) {
        const ZooT<T>& zo = p.zo[c];
        const T I = c ? M : Z;
        const int N = c ? 4 : 3;
        const T pref[4] = {zo.pP, zo.pD, zo.pPOC, zo.pZ};
        const T tb = pis_pow(zo.b_T, Tc);
        T total_food = T(0), available = T(0), total_iron = T(0), iron_avail = T(0);
        for (int k = 0; k < N; k++) total_food += food[k] * pref[k];
        for (int k = 0; k < N; k++) available += jmax(T(0), food[k] - zo.J) * pref[k];
        const T limited = jmax(T(0), available - jmin(available / T(2), zo.thr));
        const T sg = zo.g0 * tb * limited / (zo.K + total_food);
        for (int k = 0; k < N; k++) total_iron += iron_q[k] * pref[k];
        for (int k = 0; k < N; k++) iron_avail += jmax(T(0), food[k] - zo.J) * pref[k] * iron_q[k];
        const T ratio = total_iron / (zo.th_fe * sg + e);
        eff[c] = jmin(T(1), ratio) * jmin(zo.e0, (T(1) - zo.sigma) * ratio);
        spec[c] = sg;
        avail[c] = available;
        gI[c] = sg * I;
        const T ff = zo.gf0 * tb;
        gfI[c] = ff * edible * I;
        gIFe[c] = iron_avail * sg / (available + e) * I;
        gfIFe[c] = ff * edible_fe * I;
        const T cf = I / (I + zo.Km);
        mort[c] = tb * I * (zo.m0 * I + zo.r * (cf + T(3) * dO2));
        const T share = sg / (available + e) * I;
        gP[c] = zo.pP * jmax(T(0), P - zo.J) * share;
        gD[c] = zo.pD * jmax(T(0), D - zo.J) * share;
        gPOC[c] = zo.pPOC * jmax(T(0), POC - zo.J) * share;
        if (c == 1) gZ_meso = zo.pZ * jmax(T(0), Z - zo.J) * share;
        fPOC[c] = ff * (POC * wPOC) * I;
        fGOC[c] = ff * (GOC * wGOC) * I;
    }
    const ZooT<T>& mi = p.zo[0];
    const ZooT<T>& me = p.zo[1];
    const T meso_lin = pis_pow(me.b_T, Tc) * me.r * (M / (M + me.Km) + T(3) * dO2) * M;   // linear_mortality
    T exc[2], inorg_exc[2], org_exc[2], nonassim[2], nonassim_fe_waste[2], nonassim_fe[2];
    for (int c = 0; c < 2; c++) {
        const ZooT<T>& zo = p.zo[c];
        const T tot = gI[c] + gfI[c];
        nonassim[c] = zo.sigma * tot;
        exc[c] = (T(1) - zo.sigma - eff[c]) * tot;
        inorg_exc[c] = zo.gamma * exc[c];
        org_exc[c] = (T(1) - zo.gamma) * exc[c];
        nonassim_fe_waste[c] = zo.sigma * (gIFe[c] + gfIFe[c]);
        const T assimilated = zo.th_fe * eff[c] * tot;
        const T total_fe = gIFe[c] + gfIFe[c];
        nonassim_fe[c] = total_fe - zo.sigma * total_fe - assimilated;
    }
    // upper trophic (mortality_waste.jl), mesozooplankton
    const T ut_waste = T(1) / (T(1) - me.e0) * me.m0 * pis_pow(me.b_T, Tc) * M * M;
    const T ut_resp_product = (T(1) - me.e0 - me.sigma) * ut_waste;
    const T ut_excretion = (T(1) - me.gamma) * ut_resp_product;
    const T ut_respiration = me.gamma * ut_resp_product;
    const T ut_dissolved_fe = me.th_fe * ut_resp_product;
    const T ut_fecal = me.sigma * ut_waste;
    const T ut_fecal_fe = ut_fecal * me.th_fe;
    const T inorganic_excretion = inorg_exc[0] + inorg_exc[1];

    // ---- bacteria (micro_and_meso.jl:85-132)
    const T zm = jmin(zmxl, zeu);
    const T Bact = (z >= zm ? T(1) : pis_pow(zm / z, p.bdepth)) * jmin(T(4), p.bZ * Z + p.bM * M);
    const T L_N = (p.K_no3_b * NH4 + p.K_nh4_b * NO3) / (p.K_no3_b * p.K_nh4_b + p.K_no3_b * NH4 + p.K_nh4_b * NO3);
    const T LBact = jmin(jmin(L_N, PO4 / (PO4 + p.K_po4_b)), Fe / (Fe + p.K_fe_b)) * (DOC / (DOC + p.K_doc_b));

    // ---- DOC (dissolved_organic_carbon.jl:56-129)
    const T doc_deg = p.lam_doc * pis_pow(p.b_doc, Tc) * LBact * Bact / p.bact_ref * DOC;
    const T phi1 = shear * (p.a_doc[0] * DOC + p.a_doc[1] * POC) * DOC;
    const T phi2 = shear * (p.a_doc[2] * GOC) * DOC;
    const T phi3 = (p.a_doc[3] * POC + p.a_doc[4] * DOC) * DOC;
    // free_iron (iron/iron.jl:25-37)
    const T ligands = jmax(T(0.6), T(0.09) * (DOC + T(40)) - T(3));
    const T Kf = t_exp(T(16.27) - T(1565.7) / jmax(Tc + T(273.15), T(5)));
    const T Dl = T(1) + Kf * ligands - Kf * Fe;
    const T Fep = (-Dl + t_sqrt(Dl * Dl + T(4) * Kf * Fe)) / (T(2) * Kf);
    const T colloidal = T(0.5) * (Fe - Fep);
    const T CgFe1 = (phi1 + phi3) * colloidal / (DOC + e);
    const T CgFe2 = phi2 * colloidal / (DOC + e);
    const T oxic = (T(1) - dO2) * doc_deg, anoxic = dO2 * doc_deg;

    // ---- particles (two_size_class.jl, iron.jl, silicate.jl, calcite.jl)
    const T pom_agg = shear * (p.a_pom[0] * POC * POC + p.a_pom[1] * POC * GOC) + p.a_pom[2] * POC * GOC + p.a_pom[3] * POC * POC;
    const T sdeg = p.lam_pom * pis_pow(p.b_pom, Tc) * (T(1) - T(0.45) * dO2);
    const T lamFe = p.lam_fe0 + p.lam_fe1 * (POC + GOC + CaCO3 + PSi);
    const T BactFe = p.mu_bact * pis_pow(p.b_pom, Tc) * LBact * p.th_bact_fe * Fe / (Fe + p.K_bact_fe) * Bact * p.kappa_bact;
    const T chi = p.chi0 * (z >= zm ? T(1) : t_exp((p.lam_fast - p.lam_slow) * (zm - z) / wGOC));
    const T lam0 = chi * p.lam_fast + (T(1) - chi) * p.lam_slow;
    const T eq = pis_pow(T(10), T(6.44) - T(968) / (Tc + T(273.15)));
    const T sat = (eq - Si) / eq;
    const T q4 = T(1) + Tc / T(400);
    const T psi_diss = lam0 * (T(0.225) * (T(1) + Tc / T(15)) * sat + T(0.775) * pis_pow(q4 * q4 * q4 * q4 * sat, T(9))) * PSi;
    const T ca_diss = p.lam_ca * pis_pow(jmax(T(0), T(1) - a[OBGC_PAUX_OMEGA]), p.n_ca) * CaCO3;

    // ---- nano/diatom coupling (nano_diatom_coupling.jl)
    const T PAR = a[OBGC_PAUX_PAR];
    const T L_CaCO3 = jmin(jmin(n.LN, Fe / (Fe + T(0.05))), n.LPO4);
    const T R = p.rain0 * L_CaCO3 * jmax(T(1), P / T(2)) * (jmax(T(0), PAR - T(1)) / (T(4) + PAR)) * (T(30) / (T(30) + PAR)) *
                jmax(T(0), Tc / (Tc + T(0.1))) * (T(1) + t_exp(-(Tc - T(10)) * (Tc - T(10)) / T(25))) *
                jmin(T(1), T(-50) / zmxl);
    const T thP = PFe / (P + e), thD = DFe / (D + e);
    const T grazP = gP[0] + gP[1], grazD = gD[0] + gD[1];
    const T ca_prod = R * (mi.eta * gP[0] + me.eta * gP[1] + (n.lin + n.quad) / T(2));
    const T psi_prod = (grazD + d.lin + d.quad) * (DSi / (D + e));
    const T tg_POC = gPOC[0] + gPOC[1] + fPOC[0] + fPOC[1];
    const T tg_GOC = fGOC[0] + fGOC[1];

    // ---- nitrogen (nitrate_ammonia.jl:52-88)
    const T nitrif = p.lam_nitrif * NH4 / (T(1) + a[OBGC_PAUX_MLPAR]) * (T(1) - dO2);
    const T fix_limit = n.LN >= T(0.8) ? T(0.01) : T(1) - n.LN;
    const T fixation = p.N_fix * jmax(T(0), n.mu_i - T(2.15)) * fix_limit *
                       jmin(Fe / (Fe + p.K_fe_fix), PO4 / (PO4 + p.K_po4_fix)) * (T(1) - t_exp(-PAR / p.E_fix));

    // ---- tendencies
    const PiscesPhytoState<T>* cl[2] = {&n, &d};
    for (int c = 0; c < 2; c++) {
        const PhytoT<T>& ph = p.ph[c];
        const PiscesPhytoState<T>& s = *cl[c];
        const T graz = c ? grazD : grazP;
        const T death = s.lin + s.quad;
        const int base = c ? OBGC_PIS_D : OBGC_PIS_P;
        G[base] = (T(1) - ph.delta) * s.muI - death - graz;
        const T chl_growth = (T(1) - ph.delta) * T(12) * (ph.th0_chl + (ph.th1_chl - ph.th0_chl) * rho[c]) * s.mu * s.I;
        G[base + 1] = chl_growth - (death + graz) * (s.IChl / (T(12) * s.I + e)) * T(12);
        G[base + 2] = s.uFe - (death + graz) * (s.IFe / (s.I + e));
    }
    G[OBGC_PIS_DSI] = up_si - ((d.lin + d.quad) + grazD) * (DSi / (D + e));
    G[OBGC_PIS_Z] = eff[0] * (gI[0] + gfI[0]) - mort[0] - gZ_meso;
    G[OBGC_PIS_M] = eff[1] * (gI[1] + gfI[1]) - mort[1];
    G[OBGC_PIS_DOC] = p.ph[0].delta * n.muI + p.ph[1].delta * d.muI + ut_excretion + org_exc[0] + org_exc[1] + sdeg * POC -
                      doc_deg - (phi1 + phi2 + phi3);
    G[OBGC_PIS_POC] = nonassim[0] + ((T(1) - R / T(2)) * (n.lin + n.quad) + d.lin / T(2)) + mort[0] + (phi1 + phi3) + sdeg * GOC -
                      tg_POC - pom_agg - sdeg * POC;
    G[OBGC_PIS_GOC] = nonassim[1] + (R / T(2) * (n.lin + n.quad) + d.lin / T(2) + d.quad) + meso_lin + ut_fecal + pom_agg + phi2 -
                      tg_GOC - sdeg * GOC;
    const T thS = SFe / (POC + e), thB = BFe / (GOC + e);
    G[OBGC_PIS_SFE] = nonassim_fe_waste[0] + ((T(1) - R / T(2)) * (n.lin + n.quad) * thP + d.lin * thD / T(2)) + mort[0] * mi.th_fe +
                      sdeg * BFe + lamFe * POC * Fep + p.kappa_small * BactFe + CgFe1 - tg_POC * thS - pom_agg * thS - sdeg * SFe;
    G[OBGC_PIS_BFE] = nonassim_fe_waste[1] + (R / T(2) * (n.lin + n.quad) * thP + (d.lin / T(2) + d.quad) * thD) +
                      meso_lin * me.th_fe + ut_fecal_fe + lamFe * GOC * Fep + p.kappa_large * BactFe + CgFe2 + pom_agg * thS -
                      tg_GOC * thB - sdeg * BFe;
    G[OBGC_PIS_PSI] = psi_prod - psi_diss;
    G[OBGC_PIS_CACO3] = ca_prod - ca_diss;
    G[OBGC_PIS_NO3] = nitrif + p.thN * (oxic - up_no3);
    G[OBGC_PIS_NH4] = fixation + p.thN * (anoxic + inorganic_excretion + ut_respiration - up_nh4) - nitrif;
    G[OBGC_PIS_PO4] = p.thP * (inorganic_excretion + ut_respiration + doc_deg - production);
    const T Lt = jmax(p.L_max, p.L_ratio * DOC - p.L_max);
    const T ligand_aggregation = p.scav_enh * lamFe * jmax(T(0), Fe - Lt) * Fep;
    G[OBGC_PIS_FE] = sdeg * SFe + nonassim_fe[0] + nonassim_fe[1] + ut_dissolved_fe - (n.uFe + d.uFe) - ligand_aggregation -
                     (CgFe1 + CgFe2) - lamFe * (POC + GOC) * Fep - BactFe;
    G[OBGC_PIS_SI] = psi_diss - up_si;
    G[OBGC_PIS_DIC] = inorganic_excretion + ut_respiration + doc_deg + ca_diss - ca_prod - production;
    G[OBGC_PIS_ALK] = G[OBGC_PIS_NH4] - G[OBGC_PIS_NO3] - T(2) * G[OBGC_PIS_CACO3];
    G[OBGC_PIS_O2] = p.th_resp * up_nh4 + (p.th_resp + p.th_nitrif) * up_no3 + p.th_nitrif * fixation / p.thN -
                     ((p.th_resp + p.th_nitrif) * oxic + p.th_resp * anoxic) - p.th_resp * inorganic_excretion -
                     p.th_resp * ut_respiration - p.th_nitrif * nitrif / p.thN;
}

}  // namespace obgc
