/* or_pisces.c — FP64 restatement of the reference's PISCES functors (test infrastructure).
 *
 * Follows src/Models/AdvectedPopulations/PISCES/ function by function: every tracer's tendency is
 * built the way the reference's functor for that tracer builds it, recomputing the shared terms it
 * recomputes (the GPU kernel fuses them; this file is the oracle).  Paths below are relative to
 * that directory unless they start with src/.  Quirks kept verbatim:
 *   - the growth rate calls day_length(latitude, time) (growth_rate.jl:29) where the CBM day length
 *     takes (time, latitude) (src/Utils/Utils.jl:18); the energy-assimilation ratio calls it in the
 *     right order (growth_rate.jl:144);
 *   - sinking velocities are negative (downward), so flux feeding on sinking particles is negative;
 *   - nitrogen fixation compares a rate in 1/s with 2.15 (nitrate_ammonia.jl:80) and is zero;
 *   - the bacteria cap is the literal 4 (micro_and_meso.jl:98), the GOC speed divides by 5000.
 * Zooplankton pair their food preferences with the prey (P, D, POC, Z) by position
 * (food_quality_dependant.jl:144,147 with defaults.jl:45-60); with the default preference tuples
 * (P, D, POC, Z) that is the pairing by name used here.
 */
#include <math.h>
#include <string.h>
#include "obgc_oracle.h"

#define DAY 86400.0
#define EPS0 4.9406564584124654e-324   /* eps(0.0) */

static double jmin(double a, double b) { return (a != a || b != b) ? NAN : (a < b ? a : b); }
static double jmax(double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : b); }
static double min3(double a, double b, double c) { return jmin(jmin(a, b), c); }
static double min4(double a, double b, double c, double d) { return jmin(jmin(jmin(a, b), c), d); }
static double sind(double x) { return sin(fmod(x, 360.0) * (M_PI / 180.0)); }
static double cosd(double x) { return cos(fmod(x, 360.0) * (M_PI / 180.0)); }

/* ------------------------------------------------------------------ defaults -------------- */
static void phyto_defaults(obgc_pisces_phyto* c, int diatoms) {
    memset(c, 0, sizeof(*c));
    /* MixedMondo (mixed_mondo.jl:63-85) with the class values of mixed_mondo_nano_diatoms.jl:1-30 */
    c->growth_kind = 1;                                   /* GrowthRespirationLimitedProduction */
    c->silicate_limited = diatoms;
    c->exudated_fraction = 0.05;
    c->blue_light_absorption = diatoms ? 1.6 : 2.1;
    c->green_light_absorption = diatoms ? 0.69 : 0.42;
    c->red_light_absorption = diatoms ? 0.7 : 0.4;
    c->mortality_half_saturation = 0.2;
    c->linear_mortality_rate = 0.01 / DAY;
    c->base_quadratic_mortality = 0.01 / DAY;
    c->maximum_quadratic_mortality = diatoms ? 0.03 / DAY : 0.0;
    c->minimum_chlorophyll_ratio = 0.0033;
    c->maximum_chlorophyll_ratio = diatoms ? 0.05 : 0.033;
    c->maximum_iron_ratio = 0.06;
    c->silicate_half_saturation = 2.0;
    c->enhanced_silicate_half_saturation = 20.9;
    c->optimal_silicate_ratio = 0.159;
    c->half_saturation_for_iron_uptake = diatoms ? 3.0 : 1.0;
    c->threshold_for_size_dependency = 1.0;
    c->size_ratio = 3.0;
    /* growth_rate.jl:107-115 */
    c->base_growth_rate = 0.6 / DAY;
    c->temperature_sensitivity = 1.066;
    c->dark_tolerance = (diatoms ? 4 : 3) * DAY;
    c->initial_slope_of_PI_curve = 2.0;
    c->low_light_adaptation = 0.0;
    c->basal_respiration_rate = 0.033 / DAY;
    c->reference_growth_rate = 1.0 / DAY;
    /* nutrient_limitation.jl:10-18 */
    c->minimum_ammonium_half_saturation = diatoms ? 0.039 : 0.013;
    c->minimum_nitrate_half_saturation = diatoms ? 0.39 : 0.13;
    c->minimum_phosphate_half_saturation = diatoms ? 2.4 : 0.8;
    c->optimal_iron_quota = 0.007;
    c->minimum_silicate_half_saturation = 1.0;
    c->silicate_half_saturation_parameter = 16.6;
}

static void zoo_defaults(obgc_pisces_zoo* z, int meso) {
    memset(z, 0, sizeof(*z));
    /* food_quality_dependant.jl:79-96 with the class values of defaults.jl:2-21 */
    z->temperature_sensitivity = 1.079;
    z->maximum_grazing_rate = meso ? 0.75 / DAY : 3.0 / DAY;
    z->preference_P = meso ? 0.3 : 1.0;
    z->preference_D = meso ? 1.0 : 0.5;
    z->preference_POC = meso ? 0.3 : 0.1;
    z->preference_Z = meso ? 1.0 : 0.0;
    z->food_threshold_concentration = 0.3;
    z->specific_food_threshold_concentration = 0.001;
    z->grazing_half_saturation = 20.0;
    z->maximum_flux_feeding_rate = meso ? 2e3 / 1e6 : 0.0;
    z->iron_ratio = meso ? 0.015 : 0.01;
    z->minimum_growth_efficiency = meso ? 0.35 : 0.3;
    z->non_assimilated_fraction = 0.3;
    z->mortality_half_saturation = 0.2;
    z->quadratic_mortality = meso ? 0.03 / DAY : 0.004 / DAY;
    z->linear_mortality = meso ? 0.005 / DAY : 0.03 / DAY;
    z->dissolved_excretion_fraction = 0.6;
    z->undissolved_calcite_fraction = meso ? 0.75 : 0.5;
}

void or_pisces_defaults(obgc_pisces_params* p) {
    memset(p, 0, sizeof(*p));
    phyto_defaults(&p->nano, 0);
    phyto_defaults(&p->diatoms, 1);
    p->base_rain_ratio = 0.3;
    zoo_defaults(&p->micro, 0);
    zoo_defaults(&p->meso, 1);
    /* micro_and_meso.jl:3-20 */
    p->micro_bacteria = 0.7; p->meso_bacteria = 1.4; p->maximum_bacteria = 4.0; p->bacteria_depth_exponent = 0.684;
    p->doc_half_saturation_bacteria = 417.0; p->nitrate_half_saturation_bacteria = 0.03;
    p->ammonia_half_saturation_bacteria = 0.003; p->phosphate_half_saturation_bacteria = 0.003;
    p->iron_half_saturation_bacteria = 0.01;
    /* dissolved_organic_carbon.jl:18-37 */
    p->doc_remineralisation_rate = 0.3 / DAY; p->doc_bacteria_depth_exponent = 0.684;
    p->doc_reference_bacteria = 1.0; p->doc_temperature_sensitivity = 1.066;
    const double da[5] = {0.37, 102, 3530, 5095, 114};
    for (int q = 0; q < 5; q++) p->doc_aggregation[q] = da[q] * (1e-6 / DAY);
    /* two_size_class.jl:48-86 */
    p->pom_temperature_sensitivity = 1.066; p->pom_base_breakdown_rate = 0.025 / DAY;
    const double pa[4] = {25.9, 4452, 3.3, 47.1};
    for (int q = 0; q < 4; q++) p->pom_aggregation[q] = pa[q] * (1e-6 / DAY);
    p->minimum_iron_scavenging_rate = 3e-5 / DAY; p->load_specific_iron_scavenging_rate = 0.005 / DAY;
    p->bacterial_iron_uptake_efficiency = 0.16;
    p->small_fraction_bacterial_iron = 0.12 / 0.16; p->large_fraction_bacterial_iron = 0.04 / 0.16;
    p->base_liable_silicate_fraction = 0.5;
    p->fast_dissolution_rate_of_silicate = 0.025 / DAY; p->slow_dissolution_rate_of_silicate = 0.003 / DAY;
    p->base_calcite_dissolution_rate = 0.197 / DAY; p->calcite_dissolution_exponent = 1.0;
    p->maximum_iron_ratio_in_bacteria = 0.06; p->iron_half_saturation_for_bacteria = 0.3;
    p->maximum_bacterial_growth_rate = 0.6 / DAY;
    /* nitrate_ammonia.jl:10-16 */
    p->maximum_nitrification_rate = 0.05 / DAY; p->maximum_fixation_rate = 0.013 / DAY;
    p->iron_half_saturation_for_fixation = 0.1; p->phosphate_half_saturation_for_fixation = 0.8;
    p->light_saturation_for_fixation = 50.0;
    /* simple_iron.jl:9-13, oxygen.jl:21-24 */
    p->excess_scavenging_enhancement = 1000.0; p->maximum_ligand_concentration = 0.6; p->dissolved_ligand_ratio = 0.09;
    p->ratio_for_respiration = 133.0 / 122; p->ratio_for_nitrification = 32.0 / 122;
    /* PISCES.jl:288-340, common.jl:39-44, src/Utils/Utils.jl:13-15 */
    p->first_anoxia_threshold = 6.0; p->second_anoxia_threshold = 1.0;
    p->nitrogen_redfield_ratio = 16.0 / 122; p->phosphate_redfield_ratio = 1.0 / 122;
    p->mixed_layer_shear = 1.0; p->background_shear = 0.01; p->latitude = 45.0; p->day_length_coefficient = 0.833;
    p->poc_sinking_speed = 2.0 / DAY;
    p->goc_minimum_speed = 30.0 / DAY; p->goc_maximum_speed = 200.0 / DAY; p->goc_maximum_depth = 5000.0;
    p->silicate_climatology = 7.5;
    p->open_bottom = 1;
}

/* ------------------------------------------------------------------ cell context ---------- */
typedef struct {
    const obgc_pisces_params* p;
    const double* v;         /* [OBGC_PIS_NUM] */
    const double* a;         /* [OBGC_PAUX_NUM] */
    double z, t;
} cell;

#define V(n) (c->v[OBGC_PIS_##n])
#define A(n) (c->a[OBGC_PAUX_##n])

/* CBMDayLength (src/Utils/Utils.jl:18-34) */
double or_cbm_day_length(double coefficient, double t, double phi) {
    double m = fmod(t, 365.0 * DAY);
    if (m < 0) m += 365.0 * DAY;
    const double J = floor(m / DAY);
    const double theta = 0.216310 + 2 * atan(0.9671396 * tan(0.00860 * (J - 186)));
    const double decl = asin(0.39795 * cos(theta)) * (180.0 / M_PI);
    const double L = jmax(-1.0, jmin(1.0, (sind(coefficient) + sind(phi) * sind(decl)) / (cosd(phi) * cosd(decl))));
    return (24 - 24.0 / 180 * (acos(L) * (180.0 / M_PI))) * 3600.0;
}

/* anoxia_factor (common.jl:61-66) */
static double anoxia(const cell* c, double O2) {
    const double m1 = c->p->first_anoxia_threshold, m2 = c->p->second_anoxia_threshold;
    return jmin(1, jmax(0, 0.4 * (m1 - O2) / (m2 + O2)));
}

/* ------------------------------------------------------------------ phytoplankton --------- */
typedef struct { double I, IChl, IFe; } phyto_conc;

static const obgc_pisces_phyto* phyto_of(const cell* c, int diatoms, phyto_conc* q) {
    if (diatoms) { q->I = V(D); q->IChl = V(DCHL); q->IFe = V(DFE); return &c->p->diatoms; }
    q->I = V(P); q->IChl = V(PCHL); q->IFe = V(PFE);
    return &c->p->nano;
}

/* size_factor (mixed_mondo.jl:207-215) */
static double size_factor(const obgc_pisces_phyto* ph, double I) {
    const double Im = ph->threshold_for_size_dependency, S = ph->size_ratio;
    const double I1 = jmin(I, Im), I2 = jmax(0, I - Im);
    return (I1 + S * I2) / (I1 + I2 + EPS0);
}

/* nitrogen_limitation (nutrient_limitation.jl:73) */
static double nitrogen_limitation(double N1, double N2, double K1, double K2) {
    return (K2 * N1) / (K1 * K2 + K1 * N2 + K2 * N1 + EPS0);
}

typedef struct { double L, LFe, LPO4, LN, LNO3, LNH4; } limits;

/* NitrogenIronPhosphateSilicateLimitation (nutrient_limitation.jl:20-71) */
static limits nutrient_limitation(const cell* c, int diatoms) {
    phyto_conc q;
    const obgc_pisces_phyto* ph = phyto_of(c, diatoms, &q);
    const double NO3 = V(NO3), NH4 = V(NH4), PO4 = V(PO4), Si = V(SI), Sic = A(SICLIM);
    const double thFe = q.I == 0 ? 0.0 : q.IFe / (q.I + EPS0);
    const double thChl = q.I == 0 ? 0.0 : q.IChl / (12 * q.I + EPS0);
    const double Kb = size_factor(ph, q.I);
    const double Kno = ph->minimum_nitrate_half_saturation * Kb, Knh = ph->minimum_ammonium_half_saturation * Kb;
    const double Kp = ph->minimum_phosphate_half_saturation * Kb, Ksi = ph->minimum_silicate_half_saturation * Kb;
    limits l;
    l.LNO3 = nitrogen_limitation(NO3, NH4, Kno, Knh);
    l.LNH4 = nitrogen_limitation(NH4, NO3, Knh, Kno);
    l.LN = l.LNO3 + l.LNH4;
    l.LPO4 = PO4 / (PO4 + Kp + EPS0);
    const double thm = 1000 * (0.0016 / 55.85 * 12 * thChl + 1.5 * 1.21e-5 * 14 / (55.85 * 7.625) * l.LN +
                               1.15e-4 * 14 / (55.85 * 7.625) * l.LNO3);
    l.LFe = jmin(1, jmax(0, (thFe - thm) / ph->optimal_iron_quota));
    const double pk = ph->silicate_half_saturation_parameter;
    const double KSi = Ksi + 7 * Sic * Sic / (pk * pk + Sic * Sic);
    const double LSi = ph->silicate_limited ? Si / (Si + KSi) : INFINITY;
    l.L = min4(l.LN, l.LPO4, l.LFe, LSi);
    return l;
}

/* base_production_rate (growth_rate.jl:158-165) */
static double base_production_rate(const obgc_pisces_phyto* ph, double T) {
    return ph->base_growth_rate * pow(ph->temperature_sensitivity, T);
}

static double absorbed_par(const cell* c, const obgc_pisces_phyto* ph) {
    return ph->blue_light_absorption * A(PAR1) + ph->green_light_absorption * A(PAR2) + ph->red_light_absorption * A(PAR3);
}

/* light_limitation (growth_rate.jl:77-83 and 117-124) */
static double light_limitation(const obgc_pisces_phyto* ph, double I, double IChl, double T, double PAR,
                               double day_length, double L, double alpha) {
    const double theta = IChl / (12 * I + EPS0);
    if (ph->growth_kind == 0) {
        const double mu_i = base_production_rate(ph, T);
        return 1 - exp(-alpha * theta * PAR / (day_length * mu_i * L + EPS0));
    }
    return 1 - exp(-alpha * theta * PAR / (day_length * (ph->basal_respiration_rate + ph->reference_growth_rate)));
}

/* (μ::BaseProduction)(...) (growth_rate.jl:3-45); day_length(φ, t) as the reference calls it */
static double growth_rate(const cell* c, int diatoms, double L) {
    phyto_conc q;
    const obgc_pisces_phyto* ph = phyto_of(c, diatoms, &q);
    const double T = V(T);
    const double PAR = absorbed_par(c, ph);
    const double day_length = or_cbm_day_length(c->p->day_length_coefficient, c->p->latitude, c->t);
    const double dz = jmax(0, A(ZEU) - A(ZMXL));
    const double dark_residence_time = dz * dz / A(KAPPA);
    const double mu_i = ph->base_growth_rate * pow(ph->temperature_sensitivity, T);
    const double f1 = 1.5 * day_length / (day_length + 0.5 * DAY);
    const double f2 = 1 - dark_residence_time / (dark_residence_time + ph->dark_tolerance);
    const double alpha = ph->initial_slope_of_PI_curve * (1 + ph->low_light_adaptation * exp(-PAR));
    const double fl = light_limitation(ph, q.I, q.IChl, T, PAR, day_length, L, alpha);
    return mu_i * f1 * f2 * fl * L;
}

/* production_and_energy_assimilation_absorption_ratio (growth_rate.jl:126-156) */
static void production_and_rho(const cell* c, int diatoms, double* mu, double* rho) {
    phyto_conc q;
    const obgc_pisces_phyto* ph = phyto_of(c, diatoms, &q);
    const double PAR = absorbed_par(c, ph);
    const double day_length = or_cbm_day_length(c->p->day_length_coefficient, c->t, c->p->latitude);
    const double f1 = 1.5 * day_length / (day_length + 0.5 * DAY);
    const double L = nutrient_limitation(c, diatoms).L;
    *mu = growth_rate(c, diatoms, L);
    const double mu_check = *mu / f1 * day_length;
    const double alpha = ph->initial_slope_of_PI_curve * (1 + ph->low_light_adaptation * exp(-PAR));
    *rho = 12 * mu_check * q.I / (alpha * q.IChl * PAR + EPS0) * L;
}

/* total_production (mixed_mondo.jl:169-175) */
static double total_production(const cell* c, int diatoms) {
    phyto_conc q;
    phyto_of(c, diatoms, &q);
    const double L = nutrient_limitation(c, diatoms).L;
    return growth_rate(c, diatoms, L) * q.I;
}

/* mortality (mixed_mondo.jl:137-167) */
static void phyto_mortality(const cell* c, int diatoms, double* lin, double* quad) {
    phyto_conc q;
    const obgc_pisces_phyto* ph = phyto_of(c, diatoms, &q);
    const double L = nutrient_limitation(c, diatoms).L;
    const double I = q.I;
    *lin = ph->linear_mortality_rate * I / (I + ph->mortality_half_saturation) * I;
    const double w = ph->base_quadratic_mortality + ph->maximum_quadratic_mortality * 0.25 * (1 - L * L) / (0.25 + L * L);
    const double shear = c->z < A(ZMXL) ? c->p->background_shear : c->p->mixed_layer_shear;
    *quad = shear * w * I * I;
}

/* iron_uptake (mixed_mondo.jl:177-205) */
static double iron_uptake(const cell* c, int diatoms) {
    phyto_conc q;
    const obgc_pisces_phyto* ph = phyto_of(c, diatoms, &q);
    const double d = ph->exudated_fraction, thm = ph->maximum_iron_ratio;
    const double T = V(T), Fe = V(FE);
    const double thFe = q.IFe / (q.I + EPS0);
    const limits l = nutrient_limitation(c, diatoms);
    const double mu_i = base_production_rate(ph, T);
    const double K = ph->half_saturation_for_iron_uptake * size_factor(ph, q.I);
    const double L1 = Fe / (Fe + K + EPS0);
    const double L2 = 4 - 4.5 * l.LFe / (l.LFe + 1);
    return (1 - d) * thm * L1 * L2 * jmax(0, (1 - thFe / thm) / (1.05 - thFe / thm)) * mu_i * q.I;
}

/* silicate_uptake (mixed_mondo.jl:217-248) */
static double silicate_uptake(const cell* c, int diatoms) {
    phyto_conc q;
    const obgc_pisces_phyto* ph = phyto_of(c, diatoms, &q);
    const double d = ph->exudated_fraction, K1 = ph->silicate_half_saturation, K2 = ph->enhanced_silicate_half_saturation;
    const double th0 = ph->optimal_silicate_ratio;
    const double T = V(T), Si = V(SI);
    const limits l = nutrient_limitation(c, diatoms);
    const double mu = growth_rate(c, diatoms, l.L);
    const double mu_i = base_production_rate(ph, T);
    const double L1 = Si / (Si + K1 + EPS0);
    const double L2 = c->p->latitude < 0 ? pow(Si, 3) / (pow(Si, 3) + pow(K2, 3)) : 0.0;
    const double F1 = min4(mu / (mu_i * l.L + EPS0), l.LFe, l.LPO4, l.LN);
    const double F2 = jmin(1, 2.2 * jmax(0, L1 - 0.5));
    const double th1 = th0 * L1 * jmin(5.4, (4.4 * exp(-4.23 * F1) * F2 + 1) * (1 + 2 * L2));
    return (1 - d) * th1 * mu * q.I;
}

/* uptake of NO3 / NH4 (mixed_mondo.jl:250-264) */
static double uptake_N(const cell* c, int diatoms, int ammonia) {
    const limits l = nutrient_limitation(c, diatoms);
    const double muI = total_production(c, diatoms);
    return muI * (ammonia ? l.LNH4 : l.LNO3) / (l.LN + EPS0);
}

/* ------------------------------------------------------------------ zooplankton ----------- */
static const obgc_pisces_zoo* zoo_of(const cell* c, int meso, double* I) {
    *I = meso ? V(M) : V(Z);
    return meso ? &c->p->meso : &c->p->micro;
}

/* prey (P, D, POC[, Z]) of a class and its preferences (defaults.jl:41-60) */
static int prey(const cell* c, int meso, const obgc_pisces_zoo* zo, double* food, double* pref, double* iron) {
    food[0] = V(P); food[1] = V(D); food[2] = V(POC); food[3] = V(Z);
    pref[0] = zo->preference_P; pref[1] = zo->preference_D; pref[2] = zo->preference_POC; pref[3] = zo->preference_Z;
    iron[0] = V(PFE) / (V(P) + EPS0);
    iron[1] = V(DFE) / (V(D) + EPS0);
    iron[2] = V(SFE) / (V(POC) + EPS0);
    iron[3] = c->p->micro.iron_ratio;
    return meso ? 4 : 3;
}

typedef struct { double total_specific, available, gI, e; } grazing_t;

/* grazing (food_quality_dependant.jl:126-169) */
static grazing_t zoo_grazing(const cell* c, int meso) {
    double I, food[4], pref[4], iron[4];
    const obgc_pisces_zoo* zo = zoo_of(c, meso, &I);
    const int N = prey(c, meso, zo, food, pref, iron);
    const double base = zo->maximum_grazing_rate * pow(zo->temperature_sensitivity, V(T));
    double total_food = 0, available = 0, total_iron = 0;
    for (int n = 0; n < N; n++) total_food += food[n] * pref[n];
    for (int n = 0; n < N; n++) available += jmax(0, food[n] - zo->specific_food_threshold_concentration) * pref[n];
    const double limited = jmax(0, available - jmin(available / 2, zo->food_threshold_concentration));
    grazing_t g;
    g.total_specific = base * limited / (zo->grazing_half_saturation + total_food);
    g.available = available;
    for (int n = 0; n < N; n++) total_iron += iron[n] * pref[n];
    const double ratio = total_iron / (zo->iron_ratio * g.total_specific + EPS0);
    const double quality = jmin(1, ratio);
    g.e = quality * jmin(zo->minimum_growth_efficiency, (1 - zo->non_assimilated_fraction) * ratio);
    g.gI = g.total_specific * I;
    return g;
}

/* flux_rate (two_size_class.jl:95-98): concentration x centre-interpolated sinking velocity */
static double flux_rate(const cell* c, int which) {
    switch (which) {
        case OBGC_PIS_POC: return V(POC) * A(WPOC);
        case OBGC_PIS_GOC: return V(GOC) * A(WGOC);
        case OBGC_PIS_SFE: return V(SFE) * A(WPOC);
        case OBGC_PIS_BFE: return V(BFE) * A(WGOC);
    }
    return 0.0;
}

/* flux_feeding (food_quality_dependant.jl:171-186): edible flux POC + GOC */
static double zoo_flux_feeding(const cell* c, int meso) {
    double I;
    const obgc_pisces_zoo* zo = zoo_of(c, meso, &I);
    const double sinking = flux_rate(c, OBGC_PIS_POC) + flux_rate(c, OBGC_PIS_GOC);
    return zo->maximum_flux_feeding_rate * pow(zo->temperature_sensitivity, V(T)) * sinking * I;
}

/* flux_feeding on one prey (food_quality_dependant.jl:257-270) */
static double zoo_flux_feeding_prey(const cell* c, int meso, int which) {
    double I;
    const obgc_pisces_zoo* zo = zoo_of(c, meso, &I);
    return zo->maximum_flux_feeding_rate * pow(zo->temperature_sensitivity, V(T)) * flux_rate(c, which) * I;
}

/* mortality / linear_mortality (food_quality_dependant.jl:188-224) */
static double zoo_mortality(const cell* c, int meso) {
    double I;
    const obgc_pisces_zoo* zo = zoo_of(c, meso, &I);
    const double tf = pow(zo->temperature_sensitivity, V(T));
    const double cf = I / (I + zo->mortality_half_saturation);
    return tf * I * (zo->quadratic_mortality * I + zo->linear_mortality * (cf + 3 * anoxia(c, V(O2))));
}

static double zoo_linear_mortality(const cell* c, int meso) {
    double I;
    const obgc_pisces_zoo* zo = zoo_of(c, meso, &I);
    const double tf = pow(zo->temperature_sensitivity, V(T));
    const double cf = I / (I + zo->mortality_half_saturation);
    return tf * zo->linear_mortality * (cf + 3 * anoxia(c, V(O2))) * I;
}

/* grazing of one prey (food_quality_dependant.jl:226-255) */
static double zoo_grazing_prey(const cell* c, int meso, int which) {
    double I, food[4], pref[4], iron[4];
    const obgc_pisces_zoo* zo = zoo_of(c, meso, &I);
    prey(c, meso, zo, food, pref, iron);
    const grazing_t g = zoo_grazing(c, meso);
    double P = 0, p = 0;
    switch (which) {
        case OBGC_PIS_P: P = V(P); p = zo->preference_P; break;
        case OBGC_PIS_D: P = V(D); p = zo->preference_D; break;
        case OBGC_PIS_Z: P = V(Z); p = zo->preference_Z; break;
        case OBGC_PIS_POC: P = V(POC); p = zo->preference_POC; break;
    }
    return p * jmax(0, P - zo->specific_food_threshold_concentration) * g.total_specific / (g.available + EPS0) * I;
}

/* iron_grazing / iron_flux_feeding (iron_grazing.jl:2-53) */
static double zoo_iron_grazing(const cell* c, int meso) {
    double I, food[4], pref[4], iron[4];
    const obgc_pisces_zoo* zo = zoo_of(c, meso, &I);
    const int N = prey(c, meso, zo, food, pref, iron);
    const grazing_t g = zoo_grazing(c, meso);
    double s = 0;
    for (int n = 0; n < N; n++) s += jmax(0, food[n] - zo->specific_food_threshold_concentration) * pref[n] * iron[n];
    return s * g.total_specific / (g.available + EPS0) * I;
}

static double zoo_iron_flux_feeding(const cell* c, int meso) {
    double I;
    const obgc_pisces_zoo* zo = zoo_of(c, meso, &I);
    const double sinking = flux_rate(c, OBGC_PIS_SFE) + flux_rate(c, OBGC_PIS_BFE);
    return zo->maximum_flux_feeding_rate * pow(zo->temperature_sensitivity, V(T)) * sinking * I;
}

/* grazing_waste.jl:3-70 */
static double non_assimilated_waste(const cell* c, int meso) {
    const double s = (meso ? c->p->meso : c->p->micro).non_assimilated_fraction;
    return s * (zoo_grazing(c, meso).gI + zoo_flux_feeding(c, meso));
}
static double excretion(const cell* c, int meso) {
    const double s = (meso ? c->p->meso : c->p->micro).non_assimilated_fraction;
    const grazing_t g = zoo_grazing(c, meso);
    return (1 - s - g.e) * (g.gI + zoo_flux_feeding(c, meso));
}
static double inorganic_excretion(const cell* c, int meso) {
    return (meso ? c->p->meso : c->p->micro).dissolved_excretion_fraction * excretion(c, meso);
}
static double organic_excretion(const cell* c, int meso) {
    return (1 - (meso ? c->p->meso : c->p->micro).dissolved_excretion_fraction) * excretion(c, meso);
}
static double non_assimilated_iron_waste(const cell* c, int meso) {
    const double s = (meso ? c->p->meso : c->p->micro).non_assimilated_fraction;
    return s * (zoo_iron_grazing(c, meso) + zoo_iron_flux_feeding(c, meso));
}
static double non_assimilated_iron(const cell* c, int meso) {
    const obgc_pisces_zoo* zo = meso ? &c->p->meso : &c->p->micro;
    const grazing_t g = zoo_grazing(c, meso);
    const double gf = zoo_flux_feeding(c, meso);
    const double assimilated = zo->iron_ratio * g.e * (g.gI + gf);
    const double gIFe = zoo_iron_grazing(c, meso), gfIFe = zoo_iron_flux_feeding(c, meso);
    const double lost = zo->non_assimilated_fraction * (gIFe + gfIFe);
    const double total = gIFe + gfIFe;
    return total - lost - assimilated;
}

/* mortality_waste.jl:1-41 (mesozooplankton only) */
static double upper_trophic_waste(const cell* c) {
    const obgc_pisces_zoo* zo = &c->p->meso;
    const double I = V(M);
    return 1 / (1 - zo->minimum_growth_efficiency) * zo->quadratic_mortality * pow(zo->temperature_sensitivity, V(T)) * I * I;
}
static double upper_trophic_respiration_product(const cell* c) {
    const obgc_pisces_zoo* zo = &c->p->meso;
    return (1 - zo->minimum_growth_efficiency - zo->non_assimilated_fraction) * upper_trophic_waste(c);
}
static double upper_trophic_excretion(const cell* c) {
    return (1 - c->p->meso.dissolved_excretion_fraction) * upper_trophic_respiration_product(c);
}
static double upper_trophic_respiration(const cell* c) {
    return c->p->meso.dissolved_excretion_fraction * upper_trophic_respiration_product(c);
}
static double upper_trophic_dissolved_iron(const cell* c) {
    return c->p->meso.iron_ratio * upper_trophic_respiration_product(c);
}
static double upper_trophic_fecal_production(const cell* c) {
    return c->p->meso.non_assimilated_fraction * upper_trophic_waste(c);
}
static double upper_trophic_fecal_iron_production(const cell* c) {
    return upper_trophic_fecal_production(c) * c->p->meso.iron_ratio;
}

/* bacteria_concentration / bacteria_activity (micro_and_meso.jl:85-132) */
static double bacteria_concentration(const cell* c) {
    const obgc_pisces_params* p = c->p;
    const double zm = jmin(A(ZMXL), A(ZEU));
    const double surface = jmin(4, p->micro_bacteria * V(Z) + p->meso_bacteria * V(M));
    const double depth_factor = pow(zm / c->z, p->bacteria_depth_exponent);
    return (c->z >= zm ? 1.0 : depth_factor) * surface;
}
static double bacteria_activity(const cell* c) {
    const obgc_pisces_params* p = c->p;
    const double NH4 = V(NH4), NO3 = V(NO3), PO4 = V(PO4), Fe = V(FE), DOC = V(DOC);
    const double KNO3 = p->nitrate_half_saturation_bacteria, KNH4 = p->ammonia_half_saturation_bacteria;
    const double DOC_limit = DOC / (DOC + p->doc_half_saturation_bacteria);
    const double L_N = (KNO3 * NH4 + KNH4 * NO3) / (KNO3 * KNH4 + KNO3 * NH4 + KNH4 * NO3);
    const double L_PO4 = PO4 / (PO4 + p->phosphate_half_saturation_bacteria);
    const double L_Fe = Fe / (Fe + p->iron_half_saturation_bacteria);
    return min3(L_N, L_PO4, L_Fe) * DOC_limit;
}

/* ------------------------------------------------------------------ DOC -------------------- */
/* degradation (dissolved_organic_carbon.jl:56-71) */
static double doc_degradation(const cell* c) {
    const obgc_pisces_params* p = c->p;
    const double f = pow(p->doc_temperature_sensitivity, V(T));
    return p->doc_remineralisation_rate * f * bacteria_activity(c) * bacteria_concentration(c) / p->doc_reference_bacteria * V(DOC);
}

/* aggregation (dissolved_organic_carbon.jl:73-94) */
static void doc_aggregation(const cell* c, double* total, double* f1, double* f2, double* f3) {
    const double* a = c->p->doc_aggregation;
    const double shear = c->z < A(ZMXL) ? c->p->background_shear : c->p->mixed_layer_shear;
    const double DOC = V(DOC), POC = V(POC), GOC = V(GOC);
    *f1 = shear * (a[0] * DOC + a[1] * POC) * DOC;
    *f2 = shear * (a[2] * GOC) * DOC;
    *f3 = (a[3] * POC + a[4] * DOC) * DOC;
    *total = *f1 + *f2 + *f3;
}

/* free_iron (iron/iron.jl:25-37) */
static double free_iron(const cell* c) {
    const double DOC = V(DOC), Fe = V(FE), T = V(T);
    const double ligands = jmax(0.6, 0.09 * (DOC + 40) - 3);
    const double K = exp(16.27 - 1565.7 / jmax(T + 273.15, 5));
    const double D = 1 + K * ligands - K * Fe;
    return (-D + sqrt(D * D + 4 * K * Fe)) / (2 * K);
}

/* aggregation_of_colloidal_iron (dissolved_organic_carbon.jl:96-110) */
static void colloidal_iron(const cell* c, double* total, double* c1, double* c2) {
    double t, f1, f2, f3;
    doc_aggregation(c, &t, &f1, &f2, &f3);
    const double colloidal = 0.5 * (V(FE) - free_iron(c));
    *c1 = (f1 + f3) * colloidal / (V(DOC) + EPS0);
    *c2 = f2 * colloidal / (V(DOC) + EPS0);
    *total = *c1 + *c2;
}

static double oxic_remineralisation(const cell* c) { return (1 - anoxia(c, V(O2))) * doc_degradation(c); }
static double anoxic_remineralisation(const cell* c) { return anoxia(c, V(O2)) * doc_degradation(c); }

/* ------------------------------------------------------------------ POM -------------------- */
/* aggregation (two_size_class.jl:109-125) */
static double pom_aggregation(const cell* c) {
    const double* a = c->p->pom_aggregation;
    const double shear = c->z < A(ZMXL) ? c->p->background_shear : c->p->mixed_layer_shear;
    const double POC = V(POC), GOC = V(GOC);
    return shear * (a[0] * POC * POC + a[1] * POC * GOC) + a[2] * POC * GOC + a[3] * POC * POC;
}

/* specific_degradation_rate (two_size_class.jl:127-137) */
static double specific_degradation(const cell* c) {
    const obgc_pisces_params* p = c->p;
    return p->pom_base_breakdown_rate * pow(p->pom_temperature_sensitivity, V(T)) * (1 - 0.45 * anoxia(c, V(O2)));
}

/* iron.jl:97-137 */
static double iron_scavenging_rate(const cell* c) {
    return c->p->minimum_iron_scavenging_rate + c->p->load_specific_iron_scavenging_rate * (V(POC) + V(GOC) + V(CACO3) + V(PSI));
}
static double bacterial_iron_uptake(const cell* c) {
    const obgc_pisces_params* p = c->p;
    const double mu = p->maximum_bacterial_growth_rate * pow(p->pom_temperature_sensitivity, V(T));
    const double Fe = V(FE);
    return mu * bacteria_activity(c) * p->maximum_iron_ratio_in_bacteria * Fe / (Fe + p->iron_half_saturation_for_bacteria) *
           bacteria_concentration(c) * p->bacterial_iron_uptake_efficiency;
}
static double iron_scavenging(const cell* c) {
    return iron_scavenging_rate(c) * (V(POC) + V(GOC)) * free_iron(c);
}

/* particulate silicate (silicate.jl:11-48) */
static double silicate_liable_fraction(const cell* c) {
    const obgc_pisces_params* p = c->p;
    const double zm = jmin(A(ZMXL), A(ZEU));
    return p->base_liable_silicate_fraction *
           (c->z >= zm ? 1.0
                       : exp((p->fast_dissolution_rate_of_silicate - p->slow_dissolution_rate_of_silicate) * (zm - c->z) / A(WGOC)));
}
static double silicate_dissolution(const cell* c) {
    const obgc_pisces_params* p = c->p;
    const double T = V(T), Si = V(SI);
    const double chi = silicate_liable_fraction(c);
    const double l0 = chi * p->fast_dissolution_rate_of_silicate + (1 - chi) * p->slow_dissolution_rate_of_silicate;
    const double eq = pow(10, 6.44 - 968 / (T + 273.15));
    const double sat = (eq - Si) / eq;
    const double l = l0 * (0.225 * (1 + T / 15) * sat + 0.775 * pow(pow(1 + T / 400, 4) * sat, 9));
    return l * V(PSI);
}

/* calcite_dissolution (particulate_organic_matter/calcite.jl:9-19) */
static double calcite_dissolution(const cell* c) {
    const obgc_pisces_params* p = c->p;
    return p->base_calcite_dissolution_rate * pow(jmax(0, 1 - A(OMEGA)), p->calcite_dissolution_exponent) * V(CACO3);
}

/* ------------------------------------------------------------------ coupling --------------- */
/* coccolithophore_nutrient_limitation, rain_ratio (nano_diatom_coupling.jl:57-123) */
static double rain_ratio(const cell* c) {
    const limits l = nutrient_limitation(c, 0);
    const double Fe = V(FE), T = V(T), PAR = A(PAR);
    const double L_Fe = Fe / (Fe + 0.05);
    const double L_CaCO3 = min3(l.LN, L_Fe, l.LPO4);
    const double concentration_factor = jmax(1, V(P) / 2);
    const double low_light = jmax(0, PAR - 1) / (4 + PAR);
    const double high_light = 30 / (30 + PAR);
    const double low_temperature = jmax(0, T / (T + 0.1));
    const double high_temperature = 1 + exp(-(T - 10) * (T - 10) / 25);
    const double depth_factor = jmin(1, -50 / A(ZMXL));
    return c->p->base_rain_ratio * L_CaCO3 * concentration_factor * low_light * high_light * low_temperature *
           high_temperature * depth_factor;
}

/* grazing(zoo::MicroAndMeso, prey) (micro_and_meso.jl:50-52) */
static double grazing_of(const cell* c, int which) {
    return zoo_grazing_prey(c, 0, which) + zoo_grazing_prey(c, 1, which);
}
/* total_grazing (micro_meso_zoo_coupling.jl:27-32) */
static double total_grazing(const cell* c, int which) {
    const double ff = zoo_flux_feeding_prey(c, 0, which) + zoo_flux_feeding_prey(c, 1, which);
    if (which == OBGC_PIS_GOC || which == OBGC_PIS_BFE || which == OBGC_PIS_PSI || which == OBGC_PIS_CACO3) return ff;
    return grazing_of(c, which) + ff;
}

static void mortalities(const cell* c, double* Pl, double* Pq, double* Dl, double* Dq) {
    phyto_mortality(c, 0, Pl, Pq);
    phyto_mortality(c, 1, Dl, Dq);
}

/* calcite_production (nano_diatom_coupling.jl:86-94) */
static double calcite_production(const cell* c) {
    const double R = rain_ratio(c);
    double l, q;
    phyto_mortality(c, 0, &l, &q);
    const double loss = c->p->micro.undissolved_calcite_fraction * zoo_grazing_prey(c, 0, OBGC_PIS_P) +
                        c->p->meso.undissolved_calcite_fraction * zoo_grazing_prey(c, 1, OBGC_PIS_P);
    return R * (loss + (l + q) / 2);
}

/* particulate_silicate_production (nano_diatom_coupling.jl:73-84) */
static double silicate_production(const cell* c) {
    const double th = V(DSI) / (V(D) + EPS0);
    double l, q;
    phyto_mortality(c, 1, &l, &q);
    return (grazing_of(c, OBGC_PIS_D) + l + q) * th;
}

/* nitrification / nitrogen_fixation (nitrate_ammonia.jl:52-88) */
static double nitrification(const cell* c) {
    return c->p->maximum_nitrification_rate * V(NH4) / (1 + A(MLPAR)) * (1 - anoxia(c, V(O2)));
}
static double nitrogen_fixation(const cell* c) {
    const obgc_pisces_params* p = c->p;
    const double LN = nutrient_limitation(c, 0).LN;
    const double fixation_limit = LN >= 0.8 ? 0.01 : 1 - LN;
    const double mu = base_production_rate(&p->nano, V(T));
    const double requirement = jmax(0, mu - 2.15);
    const double Fe = V(FE), PO4 = V(PO4);
    const double nutrient = jmin(Fe / (Fe + p->iron_half_saturation_for_fixation),
                                 PO4 / (PO4 + p->phosphate_half_saturation_for_fixation));
    const double light = 1 - exp(-A(PAR) / p->light_saturation_for_fixation);
    return p->maximum_fixation_rate * requirement * fixation_limit * nutrient * light;
}

/* ------------------------------------------------------------------ tendencies ------------- */
static double tendency(const cell* c, int n);

static double phyto_carbon(const cell* c, int diatoms) {
    const obgc_pisces_phyto* ph = diatoms ? &c->p->diatoms : &c->p->nano;
    const double growth = (1 - ph->exudated_fraction) * total_production(c, diatoms);   /* carbon_growth */
    double l, q;
    phyto_mortality(c, diatoms, &l, &q);
    return growth - (l + q) - grazing_of(c, diatoms ? OBGC_PIS_D : OBGC_PIS_P);
}

static double phyto_chlorophyll(const cell* c, int diatoms) {
    phyto_conc qn;
    const obgc_pisces_phyto* ph = phyto_of(c, diatoms, &qn);
    double mu, rho;
    production_and_rho(c, diatoms, &mu, &rho);
    const double growth = (1 - ph->exudated_fraction) * 12 *
                          (ph->minimum_chlorophyll_ratio + (ph->maximum_chlorophyll_ratio - ph->minimum_chlorophyll_ratio) * rho) * mu * qn.I;
    const double th = qn.IChl / (12 * qn.I + EPS0);
    double l, q;
    phyto_mortality(c, diatoms, &l, &q);
    return growth - ((l + q) + grazing_of(c, diatoms ? OBGC_PIS_D : OBGC_PIS_P)) * th * 12;
}

static double phyto_iron(const cell* c, int diatoms) {
    phyto_conc qn;
    phyto_of(c, diatoms, &qn);
    const double th = qn.IFe / (qn.I + EPS0);
    double l, q;
    phyto_mortality(c, diatoms, &l, &q);
    return iron_uptake(c, diatoms) - ((l + q) + grazing_of(c, diatoms ? OBGC_PIS_D : OBGC_PIS_P)) * th;
}

static double tendency(const cell* c, int n) {
    const obgc_pisces_params* p = c->p;
    switch (n) {
        /* mixed_mondo_nano_diatoms.jl:45-111 */
        case OBGC_PIS_P: return phyto_carbon(c, 0);
        case OBGC_PIS_D: return phyto_carbon(c, 1);
        case OBGC_PIS_PCHL: return phyto_chlorophyll(c, 0);
        case OBGC_PIS_DCHL: return phyto_chlorophyll(c, 1);
        case OBGC_PIS_PFE: return phyto_iron(c, 0);
        case OBGC_PIS_DFE: return phyto_iron(c, 1);
        case OBGC_PIS_DSI: {
            const double th = V(DSI) / (V(D) + EPS0);
            double l, q;
            phyto_mortality(c, 1, &l, &q);
            return silicate_uptake(c, 1) - ((l + q) + grazing_of(c, OBGC_PIS_D)) * th;
        }
        /* micro_and_meso.jl:36-48 with growth_death (food_quality_dependant.jl:111-117) */
        case OBGC_PIS_Z: {
            const grazing_t g = zoo_grazing(c, 0);
            return g.e * (g.gI + zoo_flux_feeding(c, 0)) - zoo_mortality(c, 0) - zoo_grazing_prey(c, 1, OBGC_PIS_Z);
        }
        case OBGC_PIS_M: {
            const grazing_t g = zoo_grazing(c, 1);
            return g.e * (g.gI + zoo_flux_feeding(c, 1)) - zoo_mortality(c, 1);
        }
        /* dissolved_organic_carbon.jl:39-54 */
        case OBGC_PIS_DOC: {
            const double exudate = p->nano.exudated_fraction * total_production(c, 0) +
                                   p->diatoms.exudated_fraction * total_production(c, 1);
            double agg, f1, f2, f3;
            doc_aggregation(c, &agg, &f1, &f2, &f3);
            return exudate + upper_trophic_excretion(c) + organic_excretion(c, 0) + organic_excretion(c, 1) +
                   specific_degradation(c) * V(POC) - doc_degradation(c) - agg;
        }
        /* particulate_organic_matter/carbon.jl:3-50 */
        case OBGC_PIS_POC: {
            double Pl, Pq, Dl, Dq, agg, f1, f2, f3;
            mortalities(c, &Pl, &Pq, &Dl, &Dq);
            const double R = rain_ratio(c);
            doc_aggregation(c, &agg, &f1, &f2, &f3);
            return non_assimilated_waste(c, 0) + ((1 - R / 2) * (Pl + Pq) + Dl / 2) + zoo_mortality(c, 0) + (f1 + f3) +
                   specific_degradation(c) * V(GOC) - total_grazing(c, OBGC_PIS_POC) - pom_aggregation(c) -
                   specific_degradation(c) * V(POC);
        }
        case OBGC_PIS_GOC: {
            double Pl, Pq, Dl, Dq, agg, f1, f2, f3;
            mortalities(c, &Pl, &Pq, &Dl, &Dq);
            const double R = rain_ratio(c);
            doc_aggregation(c, &agg, &f1, &f2, &f3);
            return non_assimilated_waste(c, 1) + (R / 2 * (Pl + Pq) + Dl / 2 + Dq) + zoo_linear_mortality(c, 1) +
                   upper_trophic_fecal_production(c) + pom_aggregation(c) + f2 - total_grazing(c, OBGC_PIS_GOC) -
                   specific_degradation(c) * V(GOC);
        }
        /* particulate_organic_matter/iron.jl:2-89 */
        case OBGC_PIS_SFE: {
            const double th = V(SFE) / (V(POC) + EPS0);
            double Pl, Pq, Dl, Dq, ct, c1, c2;
            mortalities(c, &Pl, &Pq, &Dl, &Dq);
            const double R = rain_ratio(c);
            const double thP = V(PFE) / (V(P) + EPS0), thD = V(DFE) / (V(D) + EPS0);
            colloidal_iron(c, &ct, &c1, &c2);
            return non_assimilated_iron_waste(c, 0) + ((1 - R / 2) * (Pl + Pq) * thP + Dl * thD / 2) +
                   zoo_mortality(c, 0) * p->micro.iron_ratio + specific_degradation(c) * V(BFE) +
                   iron_scavenging_rate(c) * V(POC) * free_iron(c) + p->small_fraction_bacterial_iron * bacterial_iron_uptake(c) +
                   c1 - total_grazing(c, OBGC_PIS_POC) * th - pom_aggregation(c) * th - specific_degradation(c) * V(SFE);
        }
        case OBGC_PIS_BFE: {
            const double thS = V(SFE) / (V(POC) + EPS0), thB = V(BFE) / (V(GOC) + EPS0);
            double Pl, Pq, Dl, Dq, ct, c1, c2;
            mortalities(c, &Pl, &Pq, &Dl, &Dq);
            const double R = rain_ratio(c);
            const double thP = V(PFE) / (V(P) + EPS0), thD = V(DFE) / (V(D) + EPS0);
            colloidal_iron(c, &ct, &c1, &c2);
            return non_assimilated_iron_waste(c, 1) + (R / 2 * (Pl + Pq) * thP + (Dl / 2 + Dq) * thD) +
                   zoo_linear_mortality(c, 1) * p->meso.iron_ratio + upper_trophic_fecal_iron_production(c) +
                   iron_scavenging_rate(c) * V(GOC) * free_iron(c) + p->large_fraction_bacterial_iron * bacterial_iron_uptake(c) +
                   c2 + pom_aggregation(c) * thS - total_grazing(c, OBGC_PIS_GOC) * thB - specific_degradation(c) * V(BFE);
        }
        /* particulate_organic_matter/silicate.jl:1-9, calcite.jl:1-7 */
        case OBGC_PIS_PSI: return silicate_production(c) - silicate_dissolution(c);
        case OBGC_PIS_CACO3: return calcite_production(c) - calcite_dissolution(c);
        /* nitrogen/nitrate_ammonia.jl:22-50 */
        case OBGC_PIS_NO3: {
            const double uptake = uptake_N(c, 0, 0) + uptake_N(c, 1, 0);
            return nitrification(c) + p->nitrogen_redfield_ratio * (oxic_remineralisation(c) - uptake);
        }
        case OBGC_PIS_NH4: {
            const double uptake = uptake_N(c, 0, 1) + uptake_N(c, 1, 1);
            const double waste = inorganic_excretion(c, 0) + inorganic_excretion(c, 1);
            return nitrogen_fixation(c) +
                   p->nitrogen_redfield_ratio * (anoxic_remineralisation(c) + waste + upper_trophic_respiration(c) - uptake) -
                   nitrification(c);
        }
        /* phosphate.jl:21-33 */
        case OBGC_PIS_PO4: {
            const double production = total_production(c, 0) + total_production(c, 1);
            const double waste = inorganic_excretion(c, 0) + inorganic_excretion(c, 1);
            return p->phosphate_redfield_ratio * (waste + upper_trophic_respiration(c) + doc_degradation(c) - production);
        }
        /* iron/simple_iron.jl:19-53 */
        case OBGC_PIS_FE: {
            const double Fe = V(FE);
            const double lFe = iron_scavenging_rate(c);
            const double Fep = free_iron(c);
            const double Lt = jmax(p->maximum_ligand_concentration, p->dissolved_ligand_ratio * V(DOC) - p->maximum_ligand_concentration);
            const double ligand_aggregation = p->excess_scavenging_enhancement * lFe * jmax(0, Fe - Lt) * Fep;
            double ct, c1, c2;
            colloidal_iron(c, &ct, &c1, &c2);
            const double consumption = iron_uptake(c, 0) + iron_uptake(c, 1);
            const double waste = non_assimilated_iron(c, 0) + non_assimilated_iron(c, 1);
            return specific_degradation(c) * V(SFE) + waste + upper_trophic_dissolved_iron(c) - consumption -
                   ligand_aggregation - ct - iron_scavenging(c) - bacterial_iron_uptake(c);
        }
        /* silicate.jl:20-26 */
        case OBGC_PIS_SI: return silicate_dissolution(c) - silicate_uptake(c, 1);
        /* inorganic_carbon.jl:32-58 */
        case OBGC_PIS_DIC: {
            const double waste = inorganic_excretion(c, 0) + inorganic_excretion(c, 1);
            const double production = total_production(c, 0) + total_production(c, 1);
            return waste + upper_trophic_respiration(c) + doc_degradation(c) + calcite_dissolution(c) -
                   calcite_production(c) - production;
        }
        case OBGC_PIS_ALK:
            return tendency(c, OBGC_PIS_NH4) - tendency(c, OBGC_PIS_NO3) - 2 * tendency(c, OBGC_PIS_CACO3);
        /* oxygen.jl:30-51 */
        case OBGC_PIS_O2: {
            const double tr = p->ratio_for_respiration, tn = p->ratio_for_nitrification;
            const double zooplankton = tr * (inorganic_excretion(c, 0) + inorganic_excretion(c, 1));
            const double upper = tr * upper_trophic_respiration(c);
            const double remin = (tr + tn) * oxic_remineralisation(c) + tr * anoxic_remineralisation(c);
            const double nh4 = tr * (uptake_N(c, 0, 1) + uptake_N(c, 1, 1));
            const double no3 = (tr + tn) * (uptake_N(c, 0, 0) + uptake_N(c, 1, 0));
            const double nitrif = tn * nitrification(c) / p->nitrogen_redfield_ratio;
            const double fixation = tn * nitrogen_fixation(c) / p->nitrogen_redfield_ratio;
            return nh4 + no3 + fixation - remin - zooplankton - upper - nitrif;
        }
    }
    return 0.0;
}

double or_pisces_tendency(const obgc_pisces_params* p, int n, const double* values, const double* aux, double z, double t) {
    cell c = {p, values, aux, z, t};
    return tendency(&c, n);
}

void or_pisces_tendencies(const obgc_pisces_params* p, const double* values, const double* aux, double z, double t, double* G) {
    cell c = {p, values, aux, z, t};
    for (int n = 0; n < OBGC_PIS_NUM_BGC; n++) G[n] = tendency(&c, n);
}

/* ------------------------------------------------------------------ update_state pieces ---- */
/* DepthDependantSinkingSpeed at the z-faces of a column (common.jl:46-56): face k takes the
 * centre depth of cell k; the top face is zero. */
void or_pisces_goc_speed(const obgc_pisces_params* p, int Nz, const double* zc, double zmxl, double zeu, double* w_faces) {
    for (int k = 0; k < Nz; k++)
        w_faces[k] = -p->goc_minimum_speed + (p->goc_maximum_speed - p->goc_minimum_speed) * jmin(0, zc[k] - jmin(zmxl, zeu)) / 5000;
    w_faces[Nz] = 0.0;
}

/* _compute_mixed_layer_mean! (mean_mixed_layer_properties.jl:25-46) on one column (bottom first) */
double or_mixed_layer_mean(int Nz, const double* zf, const double* C, double zmxl) {
    double sum = 0, depth = 0;
    for (int k = Nz - 1; k >= 0; k--) {
        const double zk = zf[k], zk1 = zf[k + 1];
        const double dzk = zk1 - zk;
        const double dzk1 = zk1 > zmxl ? zk1 - zmxl : 0.0;
        const double dz = zk >= zmxl ? dzk : dzk1;
        sum += C[k] * dz;
        depth += dz;
    }
    return sum / depth;
}

/* conserved_tracers(::PISCES) (coupling_utils.jl:11-33): carbon, iron, phosphate, silicon,
 * nitrogen groups as slots of the PISCES tracer order. */
int or_pisces_conserved_groups(const obgc_pisces_params* p, int32_t* gn, int32_t* gslot, double* gfac) {
    const int carbon[9] = {OBGC_PIS_P, OBGC_PIS_D, OBGC_PIS_Z, OBGC_PIS_M, OBGC_PIS_DOC, OBGC_PIS_POC, OBGC_PIS_GOC,
                           OBGC_PIS_DIC, OBGC_PIS_CACO3};
    const int iron[7] = {OBGC_PIS_PFE, OBGC_PIS_DFE, OBGC_PIS_Z, OBGC_PIS_M, OBGC_PIS_SFE, OBGC_PIS_BFE, OBGC_PIS_FE};
    const double iron_f[7] = {1, 1, p->micro.iron_ratio, p->meso.iron_ratio, 1, 1, 1};
    const int phos[8] = {OBGC_PIS_P, OBGC_PIS_D, OBGC_PIS_Z, OBGC_PIS_M, OBGC_PIS_DOC, OBGC_PIS_POC, OBGC_PIS_GOC, OBGC_PIS_PO4};
    const int sil[3] = {OBGC_PIS_DSI, OBGC_PIS_SI, OBGC_PIS_PSI};
    const int nit[9] = {OBGC_PIS_NH4, OBGC_PIS_NO3, OBGC_PIS_P, OBGC_PIS_D, OBGC_PIS_Z, OBGC_PIS_M, OBGC_PIS_DOC,
                        OBGC_PIS_POC, OBGC_PIS_GOC};
    const double tP = p->phosphate_redfield_ratio, tN = p->nitrogen_redfield_ratio;
    int g = 0;
    gn[g] = 9; for (int m = 0; m < 9; m++) { gslot[g * OR_MAX_GROUP + m] = carbon[m]; gfac[g * OR_MAX_GROUP + m] = 1; } g++;
    gn[g] = 7; for (int m = 0; m < 7; m++) { gslot[g * OR_MAX_GROUP + m] = iron[m]; gfac[g * OR_MAX_GROUP + m] = iron_f[m]; } g++;
    gn[g] = 8; for (int m = 0; m < 8; m++) { gslot[g * OR_MAX_GROUP + m] = phos[m]; gfac[g * OR_MAX_GROUP + m] = m < 7 ? tP : 1; } g++;
    gn[g] = 3; for (int m = 0; m < 3; m++) { gslot[g * OR_MAX_GROUP + m] = sil[m]; gfac[g * OR_MAX_GROUP + m] = 1; } g++;
    gn[g] = 9; for (int m = 0; m < 9; m++) { gslot[g * OR_MAX_GROUP + m] = nit[m]; gfac[g * OR_MAX_GROUP + m] = m < 2 ? 1 : tN; } g++;
    return g;
}
