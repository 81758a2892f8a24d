/*
 * or_npd.c — TEST INFRASTRUCTURE (the oracle).  FP64 restatement of the NutrientsPlanktonDetritus
 * tracer functors, one reference function per C function, in the reference's evaluation order.
 * Files followed (src/Models/AdvectedPopulations/NutrientsPlanktonDetritus/):
 *   nutrients.jl, plankton.jl, detritus.jl, carbonate_system.jl, oxygen.jl, constructors.jl,
 *   NutrientsPlanktonDetritus.jl, and src/Utils/sinking_velocity_fields.jl.
 */
#include <math.h>
#include <float.h>
#include <string.h>
#include "obgc_oracle.h"

#define DAY 86400.0

/* Julia eps(x) for Float64: spacing of |x| (base/float.jl); eps(0.0) = nextfloat(0.0). */
static double jl_eps(double x) {
    double a = fabs(x);
    if (!isfinite(a)) return NAN;
    if (a < DBL_MIN) return DBL_TRUE_MIN;
    int e;
    frexp(a, &e);                     /* a = m * 2^e, m in [0.5, 1) */
    return ldexp(DBL_EPSILON, e - 1); /* 2^(exponent(a)) * eps     */
}

/* constructors.jl:65-96 (LOBSTER) and :177-227 (NPZD); defaults from the @kwdef structs. */
int or_npd_preset(int preset, obgc_npd_params* o) {
    memset(o, 0, sizeof(*o));
    o->nutrients = OBGC_NUT_NITRATE_AMMONIA;
    o->detritus = OBGC_DET_TWO_PARTICLE;
    o->carbonate_system = 0;
    o->oxygen = 0;
    o->light_limitation = OBGC_LIGHT_MONDO;
    o->has_temperature_coefficient = 0;
    o->phytoplankton_mortality_formulation = OBGC_QUADRATIC;
    o->grazing_concentration_formulation = OBGC_QUADRATIC;
    o->open_bottom = 1;
    o->nitrification_rate = 5.8e-7;                      /* nutrients.jl:17 */
    o->nitrate_half_saturation = 0.7;                    /* plankton.jl:20-54 */
    o->ammonia_half_saturation = 0.001;
    o->iron_half_saturation = 2e-4;
    o->nitrate_ammonia_inhibition = 3.0;
    o->light_half_saturation = 33.0;
    o->phytoplankton_maximum_growth_rate = 2.42e-5;
    o->iron_ratio = 4.6375e-5;
    o->phytoplankton_exudation_fraction = 0.05;
    o->ammonia_fraction_of_exudate = 0.75;
    o->temperature_coefficient = 0.0;
    o->phytoplankton_mortality_rate = 5.8e-7;
    o->zooplankton_mortality_rate = 2.31e-6;
    o->zooplankton_excretion_rate = 5.8e-7;
    o->phytoplankton_solid_waste_fraction = 1.0;
    o->excretion_inorganic_fraction = 0.5;
    o->preference_for_phytoplankton = 0.5;
    o->maximum_grazing_rate = 9.26e-6;
    o->grazing_half_saturation = 1.0;
    o->zooplankton_assimilation_fraction = 0.7;
    o->zooplankton_calcite_dissolution = 0.3;
    o->redfield_ratio = 6.56;
    o->carbon_calcite_ratio = 0.1;
    o->zooplankton_gut_calcite_dissolution = 0.3;
    o->phytoplankton_chlorophyll_ratio = 1.31;
    o->phytoplankton_sinking_speed = 0.0;                /* plankton.jl:66-67 */
    o->zooplankton_sinking_speed = 0.0;
    o->remineralisation_inorganic_fraction = 0.0;        /* detritus.jl:26-36 */
    o->small_remineralisation_rate = 5.88e-7;
    o->large_remineralisation_rate = 5.88e-7;
    o->dissolved_remineralisation_rate = 3.86e-7;
    o->small_solid_waste_fraction = 0.5;
    o->detritus_redfield_ratio = 6.56;
    o->small_particle_sinking_speed = 3.47e-5;           /* detritus.jl:222-223 */
    o->large_particle_sinking_speed = 200 / DAY;
    o->detritus_remineralisation_rate = 0.1213 / DAY;    /* detritus.jl:265-273 */
    o->small_particle_fraction = 0.5;
    o->detritus_sinking_speed = 2.7489 / DAY;
    o->respiration_oxygen_nitrogen_ratio = 10.75;        /* oxygen.jl:15-16 */
    o->nitrification_oxygen_nitrogen_ratio = 2.0;
    if (preset == OBGC_PRESET_LOBSTER) return 0;
    if (preset != OBGC_PRESET_NPZD) return -1;
    o->nutrients = OBGC_NUT_NUTRIENT;
    o->detritus = OBGC_DET_SINGLE;
    o->nitrate_half_saturation = 2.3868;
    o->phytoplankton_maximum_growth_rate = 0.6989 / DAY;
    o->phytoplankton_exudation_fraction = 0.0;
    o->has_temperature_coefficient = 1;
    o->temperature_coefficient = 1.88;
    o->phytoplankton_mortality_formulation = OBGC_LINEAR;
    o->phytoplankton_mortality_rate = (0.066 + 0.0101) / DAY;
    o->preference_for_phytoplankton = 1.0;
    o->grazing_concentration_formulation = OBGC_QUADRATIC;
    o->grazing_half_saturation = 0.5573;
    o->zooplankton_mortality_rate = 0.3395 / DAY;
    o->zooplankton_excretion_rate = 0.0102 / DAY;
    o->zooplankton_assimilation_fraction = 0.9116;
    o->phytoplankton_sinking_speed = 0.2551 / DAY;
    o->excretion_inorganic_fraction = 1.0;
    o->phytoplankton_solid_waste_fraction = 0.0101 / (0.066 + 0.0101);
    o->maximum_grazing_rate = 2.1522 / DAY;
    o->light_limitation = OBGC_LIGHT_ANALYTICAL;
    o->light_half_saturation = (0.6989 / DAY) / (0.1953 / DAY);
    return 0;
}

/* NutrientsPlanktonDetritus.jl:69-74 with the component lists of nutrients.jl:20,45,83,
 * plankton.jl:80, detritus.jl:39,83,293, carbonate_system.jl:47, oxygen.jl:19. */
int or_npd_required_tracers(const obgc_npd_params* p, int32_t* names, int cap) {
    int32_t tmp[32];
    int n = 0;
    switch (p->nutrients) {
        case OBGC_NUT_NITRATE_AMMONIA: tmp[n++] = OBGC_NO3; tmp[n++] = OBGC_NH4; break;
        case OBGC_NUT_NITRATE_AMMONIA_IRON: tmp[n++] = OBGC_NO3; tmp[n++] = OBGC_NH4; tmp[n++] = OBGC_FE; break;
        case OBGC_NUT_NUTRIENT: tmp[n++] = OBGC_N; break;
        default: return -1;
    }
    tmp[n++] = OBGC_P; tmp[n++] = OBGC_Z;
    if (p->has_temperature_coefficient) tmp[n++] = OBGC_T;
    switch (p->detritus) {
        case OBGC_DET_TWO_PARTICLE: tmp[n++] = OBGC_SPOM; tmp[n++] = OBGC_BPOM; tmp[n++] = OBGC_DOM; break;
        case OBGC_DET_VARIABLE_REDFIELD:
            tmp[n++] = OBGC_SPOC; tmp[n++] = OBGC_BPOC; tmp[n++] = OBGC_DOC;
            tmp[n++] = OBGC_SPON; tmp[n++] = OBGC_BPON; tmp[n++] = OBGC_DON; break;
        case OBGC_DET_SINGLE: tmp[n++] = OBGC_D; break;
        case OBGC_DET_NONE: break;
        default: return -1;
    }
    if (p->carbonate_system) { tmp[n++] = OBGC_DIC; tmp[n++] = OBGC_ALK; }
    if (p->oxygen) tmp[n++] = OBGC_O2;
    if (n > cap) return -1;
    memcpy(names, tmp, sizeof(int32_t) * n);
    return n;
}

/* ------------------------------------------------------------------ plankton.jl ---- */
static double mortality(int form, double X, double m) { return form == OBGC_LINEAR ? m * X : m * (X * X); }
static double concentration_limit(int form, double X, double k) {
    return form == OBGC_LINEAR ? X / (X + k) : (X * X) / (X * X + k * k);
}

/* detritus.jl:41-57,103-119,295-296,308 */
static double small_particulate_concentration(const obgc_npd_params* p, const double* v) {
    switch (p->detritus) {
        case OBGC_DET_TWO_PARTICLE: return v[OBGC_SPOM];
        case OBGC_DET_VARIABLE_REDFIELD: return v[OBGC_SPON];
        case OBGC_DET_SINGLE: return v[OBGC_D] * p->small_particle_fraction;
        default: return 0.0;
    }
}
static double large_particulate_concentration(const obgc_npd_params* p, const double* v) {
    return p->detritus == OBGC_DET_TWO_PARTICLE ? v[OBGC_BPOM] : v[OBGC_BPON];
}
static double dissolved_organic_nitrogen(const obgc_npd_params* p, const double* v) {
    return p->detritus == OBGC_DET_TWO_PARTICLE ? v[OBGC_DOM] : v[OBGC_DON];
}
static double small_particulate_carbon_concentration(const obgc_npd_params* p, const double* v) {
    return p->detritus == OBGC_DET_TWO_PARTICLE ? v[OBGC_SPOM] * p->detritus_redfield_ratio : v[OBGC_SPOC];
}
static double large_particulate_carbon_concentration(const obgc_npd_params* p, const double* v) {
    return p->detritus == OBGC_DET_TWO_PARTICLE ? v[OBGC_BPOM] * p->detritus_redfield_ratio : v[OBGC_BPOC];
}
static double dissolved_organic_carbon(const obgc_npd_params* p, const double* v) {
    return p->detritus == OBGC_DET_TWO_PARTICLE ? v[OBGC_DOM] * p->detritus_redfield_ratio : v[OBGC_DOC];
}

/* plankton.jl:393-397 */
static double weighted_phytoplankton_preference(const obgc_npd_params* p, double P, double sPOM) {
    double pt = p->preference_for_phytoplankton;
    return pt * P / (pt * P + (1 - pt) * sPOM + DBL_TRUE_MIN);
}

/* plankton.jl:118-135 */
static double total_grazing(const obgc_npd_params* p, const double* v) {
    double kG = p->grazing_half_saturation, g = p->maximum_grazing_rate;
    double Z = v[OBGC_Z], P = v[OBGC_P];
    double sPOM = small_particulate_concentration(p, v);
    double pp = weighted_phytoplankton_preference(p, P, sPOM);
    double food = pp * P + (1 - pp) * sPOM;
    double L = concentration_limit(p->grazing_concentration_formulation, food, kG);
    return g * L * Z;
}

/* plankton.jl:352-369 */
static double grazing_P(const obgc_npd_params* p, const double* v) {
    double kG = p->grazing_half_saturation, g = p->maximum_grazing_rate;
    double Z = v[OBGC_Z], P = v[OBGC_P];
    double sPOM = small_particulate_concentration(p, v);
    double pp = weighted_phytoplankton_preference(p, P, sPOM);
    double food = pp * P + (1 - pp) * sPOM;
    double L = concentration_limit(p->grazing_concentration_formulation, food, kG);
    return g * pp * L * P / (food + jl_eps(food)) * Z;
}

/* plankton.jl:371-388 (Val sPOM / sPON / D) */
static double grazing_sPOM(const obgc_npd_params* p, const double* v) {
    double kG = p->grazing_half_saturation, g = p->maximum_grazing_rate;
    double Z = v[OBGC_Z], P = v[OBGC_P];
    double sPOM = small_particulate_concentration(p, v);
    double pp = weighted_phytoplankton_preference(p, P, sPOM);
    double food = pp * P + (1 - pp) * sPOM;
    double L = concentration_limit(p->grazing_concentration_formulation, food, kG);
    return g * (1 - pp) * L * sPOM / (food + jl_eps(food)) * Z;
}

/* plankton.jl:150-188 */
static double nitrogen_limitation(const obgc_npd_params* p, const double* v) {
    double kNO3 = p->nitrate_half_saturation, kNH4 = p->ammonia_half_saturation;
    double psi = p->nitrate_ammonia_inhibition;
    double NO3 = v[OBGC_NO3], NH4 = v[OBGC_NH4];
    double nl = NO3 * exp(-psi * NH4) / (NO3 + kNO3);
    double al = fmax(0.0, NH4 / (kNH4 + NH4));
    return (nl + al) / 2;
}
static double nutrient_limitation(const obgc_npd_params* p, const double* v) {
    switch (p->nutrients) {
        case OBGC_NUT_NITRATE_AMMONIA: return nitrogen_limitation(p, v);
        case OBGC_NUT_NITRATE_AMMONIA_IRON: {
            double kFe = p->iron_half_saturation, Fe = v[OBGC_FE];
            double il = Fe / (kFe + Fe);
            return nitrogen_limitation(p, v) * il;
        }
        default: {
            double N = v[OBGC_N];
            return N / (N + p->nitrate_half_saturation);
        }
    }
}

/* plankton.jl:191-220 */
static double phytoplankton_growth(const obgc_npd_params* p, const double* v, double PAR) {
    double kPAR = p->light_half_saturation, mu0 = p->phytoplankton_maximum_growth_rate;
    double P = v[OBGC_P];
    double Ln = nutrient_limitation(p, v);
    double Ll = p->light_limitation == OBGC_LIGHT_MONDO ? PAR / (kPAR + PAR)
                                                         : PAR / sqrt(PAR * PAR + kPAR * kPAR);
    double Lt = p->has_temperature_coefficient ? pow(p->temperature_coefficient, v[OBGC_T] / 10) : 1.0;
    return mu0 * Ll * Ln * Lt * P;
}

/* plankton.jl:223-278 */
static double nutrient_uptake(const obgc_npd_params* p, int name, const double* v, double PAR) {
    double mu = phytoplankton_growth(p, v, PAR);
    if (name == OBGC_FE) return p->iron_ratio * mu;
    if (name == OBGC_N) return mu * (1 - p->ammonia_fraction_of_exudate * p->phytoplankton_exudation_fraction);
    double kNO3 = p->nitrate_half_saturation, kNH4 = p->ammonia_half_saturation;
    double psi = p->nitrate_ammonia_inhibition;
    double NO3 = v[OBGC_NO3], NH4 = v[OBGC_NH4];
    double nl = NO3 * exp(-psi * NH4) / (NO3 + kNO3);
    double al = fmax(0.0, NH4 / (kNH4 + NH4));
    if (name == OBGC_NO3) return mu * nl / (nl + al + DBL_TRUE_MIN);
    double waste = p->ammonia_fraction_of_exudate * p->phytoplankton_exudation_fraction * mu;
    return mu * al / (nl + al + DBL_TRUE_MIN) - waste;
}

/* plankton.jl:280-289 */
static double phytoplankton_primary_production(const obgc_npd_params* p, const double* v, double PAR) {
    double a = p->ammonia_fraction_of_exudate, g = p->phytoplankton_exudation_fraction;
    double rho = p->carbon_calcite_ratio, R = p->redfield_ratio;
    double muP = phytoplankton_growth(p, v, PAR);
    return (1 + rho * (1 - g) - a * g) * muP * R;
}

/* plankton.jl:292-349 */
static double plankton_inorganic_nitrogen_waste(const obgc_npd_params* p, const double* v) {
    double nuP = mortality(p->phytoplankton_mortality_formulation, v[OBGC_P], p->phytoplankton_mortality_rate);
    return p->excretion_inorganic_fraction * p->zooplankton_excretion_rate * v[OBGC_Z]
         + (1 - p->phytoplankton_solid_waste_fraction) * nuP;
}
static double plankton_organic_nitrogen_waste(const obgc_npd_params* p, const double* v, double PAR) {
    double muP = phytoplankton_growth(p, v, PAR);
    return (1 - p->ammonia_fraction_of_exudate) * p->phytoplankton_exudation_fraction * muP
         + (1 - p->excretion_inorganic_fraction) * p->zooplankton_excretion_rate * v[OBGC_Z];
}
static double solid_waste(const obgc_npd_params* p, const double* v) {
    double Z = v[OBGC_Z];
    double G = total_grazing(p, v);
    double nuP = mortality(p->phytoplankton_mortality_formulation, v[OBGC_P], p->phytoplankton_mortality_rate);
    return (1 - p->zooplankton_assimilation_fraction) * G + p->phytoplankton_solid_waste_fraction * nuP
         + p->zooplankton_mortality_rate * (Z * Z);
}

/* plankton.jl:399-450 */
static double calcite_production(const obgc_npd_params* p, const double* v) {
    double R = p->redfield_ratio, rho = p->carbon_calcite_ratio, eta = p->zooplankton_gut_calcite_dissolution;
    double G = grazing_P(p, v);
    double nu = mortality(p->phytoplankton_mortality_formulation, v[OBGC_P], p->phytoplankton_mortality_rate);
    return (G * (1 - eta) + nu) * rho * R;
}
static double calcite_dissolution(const obgc_npd_params* p, const double* v) {
    double R = p->redfield_ratio, rho = p->carbon_calcite_ratio;
    double G = grazing_P(p, v);
    if (p->detritus == OBGC_DET_VARIABLE_REDFIELD)   /* generic method, :414-422 */
        return G * p->zooplankton_gut_calcite_dissolution * rho * R;
    double nu = mortality(p->phytoplankton_mortality_formulation, v[OBGC_P], p->phytoplankton_mortality_rate);
    return (G + nu) * rho * R;                        /* :429-441 */
}
static double calcite_uptake(const obgc_npd_params* p, const double* v, double PAR) {
    return 2 * p->carbon_calcite_ratio * phytoplankton_growth(p, v, PAR) * p->redfield_ratio;
}

/* nutrients.jl:154,191 */
static double nitrification(const obgc_npd_params* p, const double* v) {
    return p->nutrients == OBGC_NUT_NUTRIENT ? 0.0 : p->nitrification_rate * v[OBGC_NH4];
}

/* detritus.jl:161-207,298-302,311-317 */
static double detritus_inorganic_nitrogen_waste(const obgc_npd_params* p, const double* v, double PAR) {
    switch (p->detritus) {
        case OBGC_DET_SINGLE: return v[OBGC_D] * p->detritus_remineralisation_rate;
        case OBGC_DET_NONE: return plankton_organic_nitrogen_waste(p, v, PAR) + solid_waste(p, v);
        default: {
            double a = p->remineralisation_inorganic_fraction;
            double sm = p->small_remineralisation_rate, bm = p->large_remineralisation_rate;
            double dm = p->dissolved_remineralisation_rate;
            return a * (sm * small_particulate_concentration(p, v) + bm * large_particulate_concentration(p, v))
                 + dm * dissolved_organic_nitrogen(p, v);
        }
    }
}
static double detritus_organic_nitrogen_waste(const obgc_npd_params* p, const double* v) {
    double a = p->remineralisation_inorganic_fraction;
    double sm = p->small_remineralisation_rate, bm = p->large_remineralisation_rate;
    return (1 - a) * (sm * small_particulate_concentration(p, v) + bm * large_particulate_concentration(p, v));
}
static double detritus_inorganic_carbon_waste(const obgc_npd_params* p, const double* v, double PAR) {
    switch (p->detritus) {
        case OBGC_DET_SINGLE: return v[OBGC_D] * p->detritus_remineralisation_rate * p->detritus_redfield_ratio;
        case OBGC_DET_NONE:
            return (plankton_organic_nitrogen_waste(p, v, PAR) + solid_waste(p, v)) * p->redfield_ratio;
        default: {
            double a = p->remineralisation_inorganic_fraction;
            double sm = p->small_remineralisation_rate, bm = p->large_remineralisation_rate;
            double dm = p->dissolved_remineralisation_rate;
            return a * (sm * small_particulate_carbon_concentration(p, v) + bm * large_particulate_carbon_concentration(p, v))
                 + dm * dissolved_organic_carbon(p, v);
        }
    }
}
static double detritus_organic_carbon_waste(const obgc_npd_params* p, const double* v) {
    double a = p->remineralisation_inorganic_fraction;
    double sm = p->small_remineralisation_rate, bm = p->large_remineralisation_rate;
    return (1 - a) * (sm * small_particulate_carbon_concentration(p, v) + bm * large_particulate_carbon_concentration(p, v));
}

static int has_nitrate_ammonia(const obgc_npd_params* p) {
    return p->nutrients == OBGC_NUT_NITRATE_AMMONIA || p->nutrients == OBGC_NUT_NITRATE_AMMONIA_IRON;
}
static int two_particle(const obgc_npd_params* p) {
    return p->detritus == OBGC_DET_TWO_PARTICLE || p->detritus == OBGC_DET_VARIABLE_REDFIELD;
}

/* The discrete functor (bgc)(i, j, k, grid, Val(name), clock, fields, auxiliary_fields); names the
 * model has no method for fall back to zero (NutrientsPlanktonDetritus.jl:88). */
double or_npd_tendency(const obgc_npd_params* p, int name, const double* v, double PAR) {
    switch (name) {
        case OBGC_NO3:   /* nutrients.jl:156-159 */
            if (!has_nitrate_ammonia(p)) return 0.0;
            return nitrification(p, v) - nutrient_uptake(p, OBGC_NO3, v, PAR);
        case OBGC_NH4:   /* nutrients.jl:161-166 */
            if (!has_nitrate_ammonia(p)) return 0.0;
            return plankton_inorganic_nitrogen_waste(p, v) + detritus_inorganic_nitrogen_waste(p, v, PAR)
                 - nitrification(p, v) - nutrient_uptake(p, OBGC_NH4, v, PAR);
        case OBGC_FE:    /* nutrients.jl:47-48 */
            if (p->nutrients != OBGC_NUT_NITRATE_AMMONIA_IRON) return 0.0;
            return -nutrient_uptake(p, OBGC_FE, v, PAR);
        case OBGC_N:     /* nutrients.jl:185-189 */
            if (p->nutrients != OBGC_NUT_NUTRIENT) return 0.0;
            return plankton_inorganic_nitrogen_waste(p, v) + detritus_inorganic_nitrogen_waste(p, v, PAR)
                 - nutrient_uptake(p, OBGC_N, v, PAR);
        case OBGC_P: {   /* plankton.jl:92-105 */
            double g = p->phytoplankton_exudation_fraction;
            double muP = phytoplankton_growth(p, v, PAR);
            double Gp = grazing_P(p, v);
            double nu = mortality(p->phytoplankton_mortality_formulation, v[OBGC_P], p->phytoplankton_mortality_rate);
            return (1 - g) * muP - Gp - nu;
        }
        case OBGC_Z: {   /* plankton.jl:107-116 */
            double Z = v[OBGC_Z];
            double G = total_grazing(p, v);
            return p->zooplankton_assimilation_fraction * G - p->zooplankton_mortality_rate * (Z * Z)
                 - p->zooplankton_excretion_rate * Z;
        }
        case OBGC_DOM: case OBGC_DON:   /* detritus.jl:143-147 */
            if (!two_particle(p)) return 0.0;
            if ((name == OBGC_DOM) != (p->detritus == OBGC_DET_TWO_PARTICLE)) return 0.0;
            return plankton_organic_nitrogen_waste(p, v, PAR) + detritus_organic_nitrogen_waste(p, v)
                 - p->dissolved_remineralisation_rate * dissolved_organic_nitrogen(p, v);
        case OBGC_SPOM: case OBGC_SPON:  /* detritus.jl:149-153 */
            if (!two_particle(p)) return 0.0;
            if ((name == OBGC_SPOM) != (p->detritus == OBGC_DET_TWO_PARTICLE)) return 0.0;
            return p->small_solid_waste_fraction * solid_waste(p, v) - grazing_sPOM(p, v)
                 - p->small_remineralisation_rate * small_particulate_concentration(p, v);
        case OBGC_BPOM: case OBGC_BPON:  /* detritus.jl:155-158 */
            if (!two_particle(p)) return 0.0;
            if ((name == OBGC_BPOM) != (p->detritus == OBGC_DET_TWO_PARTICLE)) return 0.0;
            return (1 - p->small_solid_waste_fraction) * solid_waste(p, v)
                 - p->large_remineralisation_rate * large_particulate_concentration(p, v);
        case OBGC_SPOC:  /* detritus.jl:85-89; grazing(Val sPOC) plankton.jl:390-391 */
            if (p->detritus != OBGC_DET_VARIABLE_REDFIELD) return 0.0;
            return p->small_solid_waste_fraction * (solid_waste(p, v) * p->redfield_ratio)
                 - grazing_sPOM(p, v) * p->redfield_ratio
                 - p->small_remineralisation_rate * small_particulate_carbon_concentration(p, v);
        case OBGC_BPOC:  /* detritus.jl:91-95 */
            if (p->detritus != OBGC_DET_VARIABLE_REDFIELD) return 0.0;
            return (1 - p->small_solid_waste_fraction) * (solid_waste(p, v) * p->redfield_ratio)
                 + calcite_production(p, v)
                 - p->large_remineralisation_rate * large_particulate_carbon_concentration(p, v);
        case OBGC_DOC:   /* detritus.jl:97-101 */
            if (p->detritus != OBGC_DET_VARIABLE_REDFIELD) return 0.0;
            return p->redfield_ratio * plankton_organic_nitrogen_waste(p, v, PAR)
                 + detritus_organic_carbon_waste(p, v)
                 - p->dissolved_remineralisation_rate * dissolved_organic_carbon(p, v);
        case OBGC_D:     /* detritus.jl:282-288 */
            if (p->detritus != OBGC_DET_SINGLE) return 0.0;
            return plankton_organic_nitrogen_waste(p, v, PAR) + solid_waste(p, v) - grazing_sPOM(p, v)
                 - p->detritus_remineralisation_rate * v[OBGC_D];
        case OBGC_DIC:   /* carbonate_system.jl:49-54 */
            if (!p->carbonate_system) return 0.0;
            return -phytoplankton_primary_production(p, v, PAR)
                 + p->redfield_ratio * plankton_inorganic_nitrogen_waste(p, v)
                 + detritus_inorganic_carbon_waste(p, v, PAR)
                 + calcite_dissolution(p, v);
        case OBGC_ALK:   /* carbonate_system.jl:56-67 */
            if (!p->carbonate_system) return 0.0;
            if (p->nutrients == OBGC_NUT_NUTRIENT)
                return or_npd_tendency(p, OBGC_N, v, PAR)
                     - 2.0 * calcite_uptake(p, v, PAR) + 2.0 * calcite_dissolution(p, v);
            return or_npd_tendency(p, OBGC_NH4, v, PAR) * (1 - 1.0 / 16)
                 - or_npd_tendency(p, OBGC_NO3, v, PAR) * (1 + 1.0 / 16)
                 - 2.0 * calcite_uptake(p, v, PAR) + 2.0 * calcite_dissolution(p, v);
        case OBGC_O2: {  /* oxygen.jl:21-31; the Nutrient specialisation (:33-43) dispatches on the
                            plankton slot and is never selected, so the NH4 term uses the zero
                            fallback when there is no NH4 functor. */
            if (!p->oxygen) return 0.0;
            double Rp = p->respiration_oxygen_nitrogen_ratio, Rn = p->nitrification_oxygen_nitrogen_ratio;
            double muP = phytoplankton_growth(p, v, PAR);
            double nitrate_production = or_npd_tendency(p, OBGC_NH4, v, PAR);
            double muNH4 = nitrification(p, v);
            return Rp * muP - (Rp - Rn) * nitrate_production - Rp * muNH4;
        }
        default:
            return 0.0;
    }
}

/* biogeochemical_drift_velocity + setup_velocity_fields: w on Nz+1 faces (face f below cell f);
 * faces 0..Nz-1 set to -w0*(open ? 1 : 1 - exp(-f/2)), the top face stays 0. */
void or_npd_drift_profile(const obgc_npd_params* p, int name, int Nz, double* w, int* drifts) {
    double w0 = 0.0;
    *drifts = 0;
    if (name == OBGC_P) { w0 = p->phytoplankton_sinking_speed; *drifts = 1; }
    else if (name == OBGC_Z) { w0 = p->zooplankton_sinking_speed; *drifts = 1; }
    else if (two_particle(p) && (name == OBGC_SPOM || name == OBGC_SPON || name == OBGC_SPOC)) {
        if ((name == OBGC_SPOM) != (p->detritus == OBGC_DET_TWO_PARTICLE)) return;
        w0 = p->small_particle_sinking_speed; *drifts = 1;
    } else if (two_particle(p) && (name == OBGC_BPOM || name == OBGC_BPON || name == OBGC_BPOC)) {
        if ((name == OBGC_BPOM) != (p->detritus == OBGC_DET_TWO_PARTICLE)) return;
        w0 = p->large_particle_sinking_speed; *drifts = 1;
    } else if (p->detritus == OBGC_DET_SINGLE && name == OBGC_D) { w0 = p->detritus_sinking_speed; *drifts = 1; }
    if (!*drifts) return;
    for (int f = 0; f < Nz; f++)
        w[f] = -w0 * (p->open_bottom ? 1.0 : (1 - exp((double)(-f) / 2)));
    w[Nz] = 0.0;
}
