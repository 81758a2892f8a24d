/*
 * obgc.h — C ABI of the GB300-native OceanBioME tracer-tendency engine (libobgc.so).
 *
 * Every entry point is extern "C", takes plain pointers, sizes and POD structs, and returns an
 * int status (OBGC_OK == 0).  No exception crosses the ABI.  Device pointers are CUDA device
 * addresses on the current device; `stream` is a cudaStream_t passed as void* (NULL = default
 * stream).  Every asynchronous call is stream-ordered.  A context is single-stream and not
 * thread-safe: serialise calls on one context externally.
 *
 * Each declaration names the OceanBioME.jl (v0.17.6) interface it replaces, as file:line within
 * that project.
 */
#ifndef OBGC_H
#define OBGC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OBGC_ABI_VERSION 2

/* ---------------------------------------------------------------------------------------
 * Status codes.  Host-side errors in the reference are Julia exceptions (ArgumentError at
 * src/Light/multi_band.jl:106, src/BoxModel/boxmodel.jl:138) or `@warn` (src/Utils/solvers.jl:118);
 * here they are return codes, with a message available from obgc_last_error_message().
 * ------------------------------------------------------------------------------------- */
enum obgc_status {
    OBGC_OK = 0,
    OBGC_ERR_INVALID_ARGUMENT = 1, /* bad descriptor, size, pointer or parameter           */
    OBGC_ERR_CUDA = 2,             /* a CUDA runtime call failed                            */
    OBGC_ERR_NOT_CONVERGED = 3,    /* a root solve hit its iteration limit                  */
    OBGC_ERR_NAN = 4,              /* a NaN/Inf was detected in a result                    */
    OBGC_ERR_UNSUPPORTED = 5,      /* the model variant/grid has no fused kernel            */
    OBGC_ERR_OUT_OF_MEMORY = 6,    /* device allocation failed or budget exceeded           */
    OBGC_ERR_NO_DEVICE = 7,        /* no CUDA device is visible                             */
    OBGC_ERR_BUSY = 8,             /* service has no free slot / budget for the request     */
    OBGC_ERR_TIMEOUT = 9           /* a bounded wait expired                                */
};

/* Storage / compute precision of a field or a run. */
enum obgc_dtype { OBGC_F32 = 0, OBGC_F64 = 1 };
/* Negative-tracer modifier applied to the initial state and after every RK3 stage, as
 * Oceananigans' update_state! runs update_biogeochemical_state!(model, modifier)
 * (src/OceanBioME.jl:161-169, src/Utils/negative_tracers.jl). */
enum obgc_negatives {
    OBGC_NEGATIVES_NONE = 0,
    OBGC_NEGATIVES_SCALE = 1,  /* ScaleNegativeTracers over conserved_tracers (scale_negatives = true) */
    OBGC_NEGATIVES_ZERO = 2    /* ZeroNegativeTracers(; exclude)                                      */
};
enum obgc_precision {
    OBGC_PREC_F32 = 0,   /* FP32 state, FP32 compute                                       */
    OBGC_PREC_F64 = 1,   /* FP64 state, FP64 compute (plain FP64 path)                     */
    OBGC_PREC_MIXED = 2  /* FP64 state (RK3 accumulation), FP32 stencil/BGC compute       */
};

/* ---------------------------------------------------------------------------------------
 * Named tracer slots.  Every tendency entry point addresses tracers by these names, so the
 * caller's field order never matters.  Names follow required_biogeochemical_tracers of the
 * NutrientsPlanktonDetritus components (src/Models/AdvectedPopulations/NutrientsPlanktonDetritus/
 * nutrients.jl:20,45,83; plankton.jl:80; detritus.jl:39,83,293; carbonate_system.jl:47;
 * oxygen.jl:19).  T and S are carried (advected) and read by the carbonate chemistry.
 * ------------------------------------------------------------------------------------- */
enum obgc_tracer {
    OBGC_NO3 = 0, OBGC_NH4, OBGC_FE, OBGC_N,
    OBGC_P, OBGC_Z, OBGC_T,
    OBGC_SPOM, OBGC_BPOM, OBGC_DOM,
    OBGC_SPON, OBGC_BPON, OBGC_DON, OBGC_SPOC, OBGC_BPOC, OBGC_DOC,
    OBGC_D,
    OBGC_DIC, OBGC_ALK, OBGC_O2,
    OBGC_S,
    OBGC_NUM_NAMED
};
#define OBGC_MAX_PASSIVE 8
/* Tracer codes of the 3-D context's setters (gas exchange, forcing, sediment): a name of enum
 * obgc_tracer, or OBGC_PASSIVE(p) for passive tracer p (obgc_fields.passive[p]). */
#define OBGC_PASSIVE(p) (OBGC_NUM_NAMED + (p))

/* Component kinds of NutrientsPlanktonDetritus (NutrientsPlanktonDetritus.jl:27-33). */
enum obgc_nutrients { OBGC_NUT_NITRATE_AMMONIA = 0, OBGC_NUT_NITRATE_AMMONIA_IRON = 1, OBGC_NUT_NUTRIENT = 2 };
enum obgc_detritus  { OBGC_DET_TWO_PARTICLE = 0, OBGC_DET_VARIABLE_REDFIELD = 1, OBGC_DET_SINGLE = 2, OBGC_DET_NONE = 3 };
enum obgc_light_limitation { OBGC_LIGHT_MONDO = 0, OBGC_LIGHT_ANALYTICAL = 1 };   /* plankton.jl:216-220 */
enum obgc_formulation { OBGC_LINEAR = 0, OBGC_QUADRATIC = 1 };                      /* plankton.jl:83-90   */
enum obgc_preset { OBGC_PRESET_LOBSTER = 0, OBGC_PRESET_NPZD = 1 };                 /* constructors.jl     */

/*
 * Parameters of a NutrientsPlanktonDetritus model, field for field the @kwdef structs
 * NitrateAmmonia (nutrients.jl:16-18), PhytoZoo (plankton.jl:19-58), TwoParticleAndDissolved
 * (detritus.jl:25-37), VariableRedfieldDetritus (detritus.jl:71-81), Detritus (detritus.jl:264-270)
 * and Oxygen (oxygen.jl:14-17).  Sinking speeds are the scalar speeds that setup_velocity_fields
 * (src/Utils/sinking_velocity_fields.jl:10-35) turns into ZFaceFields, positive downwards, in m/s.
 */
typedef struct obgc_npd_params {
    int32_t nutrients;            /* enum obgc_nutrients                                     */
    int32_t detritus;             /* enum obgc_detritus                                      */
    int32_t carbonate_system;     /* 0/1: CarbonateSystem() present                          */
    int32_t oxygen;               /* 0/1: Oxygen() present                                   */
    int32_t light_limitation;     /* enum obgc_light_limitation                              */
    int32_t has_temperature_coefficient; /* 0 = `nothing` (no Q10), 1 = Q10 used             */
    int32_t phytoplankton_mortality_formulation; /* enum obgc_formulation                    */
    int32_t grazing_concentration_formulation;   /* enum obgc_formulation                    */
    int32_t open_bottom;          /* sinking fields leave through the bottom (1) or taper (0) */
    int32_t reserved0;
    /* NitrateAmmonia / NitrateAmmoniaIron */
    double nitrification_rate;
    /* PhytoZoo */
    double nitrate_half_saturation;
    double ammonia_half_saturation;
    double iron_half_saturation;
    double nitrate_ammonia_inhibition;
    double light_half_saturation;
    double phytoplankton_maximum_growth_rate;
    double iron_ratio;
    double phytoplankton_exudation_fraction;
    double ammonia_fraction_of_exudate;
    double temperature_coefficient;
    double phytoplankton_mortality_rate;
    double zooplankton_mortality_rate;
    double zooplankton_excretion_rate;
    double phytoplankton_solid_waste_fraction;
    double excretion_inorganic_fraction;
    double preference_for_phytoplankton;
    double maximum_grazing_rate;
    double grazing_half_saturation;
    double zooplankton_assimilation_fraction;
    double zooplankton_calcite_dissolution;
    double redfield_ratio;
    double carbon_calcite_ratio;
    double zooplankton_gut_calcite_dissolution;
    double phytoplankton_chlorophyll_ratio;
    double phytoplankton_sinking_speed;
    double zooplankton_sinking_speed;
    /* TwoParticleAndDissolved / VariableRedfieldDetritus */
    double remineralisation_inorganic_fraction;
    double small_remineralisation_rate;
    double large_remineralisation_rate;
    double dissolved_remineralisation_rate;
    double small_solid_waste_fraction;
    double detritus_redfield_ratio;
    double small_particle_sinking_speed;
    double large_particle_sinking_speed;
    /* Detritus (single class) */
    double detritus_remineralisation_rate;
    double small_particle_fraction;
    double detritus_sinking_speed;
    /* Oxygen */
    double respiration_oxygen_nitrogen_ratio;
    double nitrification_oxygen_nitrogen_ratio;
} obgc_npd_params;

/* ---------------------------------------------------------------------------------------------
 * PISCES (src/Models/AdvectedPopulations/PISCES).  Tracer slots in required_biogeochemical_tracers
 * order (PISCES.jl:86-98): P PChl PFe D DChl DFe DSi Z M DOC POC GOC SFe BFe PSi CaCO3 NO3 NH4 PO4 Fe
 * Si DIC Alk O2, then T and S.
 * ------------------------------------------------------------------------------------------- */
enum obgc_pisces_tracer {
    OBGC_PIS_P = 0, OBGC_PIS_PCHL, OBGC_PIS_PFE, OBGC_PIS_D, OBGC_PIS_DCHL, OBGC_PIS_DFE, OBGC_PIS_DSI,
    OBGC_PIS_Z, OBGC_PIS_M, OBGC_PIS_DOC, OBGC_PIS_POC, OBGC_PIS_GOC, OBGC_PIS_SFE, OBGC_PIS_BFE,
    OBGC_PIS_PSI, OBGC_PIS_CACO3, OBGC_PIS_NO3, OBGC_PIS_NH4, OBGC_PIS_PO4, OBGC_PIS_FE, OBGC_PIS_SI,
    OBGC_PIS_DIC, OBGC_PIS_ALK, OBGC_PIS_O2, OBGC_PIS_T, OBGC_PIS_S,
    OBGC_PIS_NUM_BGC = 24,       /* tracers with a tendency                                    */
    OBGC_PIS_NUM = 26
};
/* Auxiliary inputs of a cell (required_biogeochemical_auxiliary_fields, PISCES.jl:100-101). */
enum obgc_pisces_aux {
    OBGC_PAUX_ZMXL = 0,   /* mixed-layer depth (m, negative)                                    */
    OBGC_PAUX_ZEU,        /* euphotic depth (m, negative)                                       */
    OBGC_PAUX_SICLIM,     /* silicate climatology Si'                                          */
    OBGC_PAUX_OMEGA,      /* calcite saturation                                                 */
    OBGC_PAUX_KAPPA,      /* mean mixed-layer vertical diffusivity                              */
    OBGC_PAUX_MLPAR,      /* mean mixed-layer PAR                                               */
    OBGC_PAUX_WPOC,       /* POC sinking velocity interpolated to the cell centre (m/s, <= 0)  */
    OBGC_PAUX_WGOC,       /* GOC sinking velocity interpolated to the cell centre (m/s, <= 0)  */
    OBGC_PAUX_PAR, OBGC_PAUX_PAR1, OBGC_PAUX_PAR2, OBGC_PAUX_PAR3,
    OBGC_PAUX_NUM = 12
};

/* One MixedMondo phytoplankton class with its growth rate and nutrient limitation
 * (phytoplankton/mixed_mondo.jl:23-99, growth_rate.jl:69-124, nutrient_limitation.jl:10-18). */
typedef struct obgc_pisces_phyto {
    int32_t growth_kind;         /* 0 NutrientLimitedProduction, 1 GrowthRespirationLimitedProduction */
    int32_t silicate_limited;
    double exudated_fraction, blue_light_absorption, green_light_absorption, red_light_absorption;
    double mortality_half_saturation, linear_mortality_rate, base_quadratic_mortality, maximum_quadratic_mortality;
    double minimum_chlorophyll_ratio, maximum_chlorophyll_ratio, maximum_iron_ratio;
    double silicate_half_saturation, enhanced_silicate_half_saturation, optimal_silicate_ratio;
    double half_saturation_for_iron_uptake, threshold_for_size_dependency, size_ratio;
    double base_growth_rate, temperature_sensitivity, dark_tolerance, initial_slope_of_PI_curve,
           low_light_adaptation, basal_respiration_rate, reference_growth_rate;
    double minimum_ammonium_half_saturation, minimum_nitrate_half_saturation,
           minimum_phosphate_half_saturation, optimal_iron_quota, minimum_silicate_half_saturation,
           silicate_half_saturation_parameter;
} obgc_pisces_phyto;

/* One QualityDependantZooplankton class (zooplankton/food_quality_dependant.jl:11-108). */
typedef struct obgc_pisces_zoo {
    double temperature_sensitivity, maximum_grazing_rate;
    double preference_P, preference_D, preference_POC, preference_Z;
    double food_threshold_concentration, specific_food_threshold_concentration, grazing_half_saturation;
    double maximum_flux_feeding_rate, iron_ratio, minimum_growth_efficiency, non_assimilated_fraction;
    double mortality_half_saturation, quadratic_mortality, linear_mortality;
    double dissolved_excretion_fraction, undissolved_calcite_fraction;
} obgc_pisces_zoo;

typedef struct obgc_pisces_params {
    obgc_pisces_phyto nano, diatoms;
    double base_rain_ratio;                       /* NanoAndDiatoms                         */
    obgc_pisces_zoo micro, meso;
    /* MicroAndMeso bacteria (zooplankton/micro_and_meso.jl:3-20) */
    double micro_bacteria, meso_bacteria, maximum_bacteria, bacteria_depth_exponent;
    double doc_half_saturation_bacteria, nitrate_half_saturation_bacteria, ammonia_half_saturation_bacteria,
           phosphate_half_saturation_bacteria, iron_half_saturation_bacteria;
    /* DissolvedOrganicCarbon (dissolved_organic_carbon.jl:9-37) */
    double doc_remineralisation_rate, doc_bacteria_depth_exponent, doc_reference_bacteria,
           doc_temperature_sensitivity, doc_aggregation[5];
    /* TwoCompartmentCarbonIronParticles (two_size_class.jl:17-86) */
    double pom_temperature_sensitivity, pom_base_breakdown_rate, pom_aggregation[4];
    double minimum_iron_scavenging_rate, load_specific_iron_scavenging_rate, bacterial_iron_uptake_efficiency;
    double small_fraction_bacterial_iron, large_fraction_bacterial_iron, base_liable_silicate_fraction;
    double fast_dissolution_rate_of_silicate, slow_dissolution_rate_of_silicate;
    double base_calcite_dissolution_rate, calcite_dissolution_exponent;
    double maximum_iron_ratio_in_bacteria, iron_half_saturation_for_bacteria, maximum_bacterial_growth_rate;
    /* NitrateAmmonia (nitrogen/nitrate_ammonia.jl:10-16) */
    double maximum_nitrification_rate, maximum_fixation_rate, iron_half_saturation_for_fixation,
           phosphate_half_saturation_for_fixation, light_saturation_for_fixation;
    /* SimpleIron (iron/simple_iron.jl:9-13) */
    double excess_scavenging_enhancement, maximum_ligand_concentration, dissolved_ligand_ratio;
    /* Oxygen (oxygen.jl:21-24) */
    double ratio_for_respiration, ratio_for_nitrification;
    /* PISCES (PISCES.jl:288-340) */
    double first_anoxia_threshold, second_anoxia_threshold, nitrogen_redfield_ratio, phosphate_redfield_ratio;
    double mixed_layer_shear, background_shear, latitude, day_length_coefficient;
    /* sinking: POC at a constant speed, GOC by DepthDependantSinkingSpeed (common.jl:39-56) */
    double poc_sinking_speed, goc_minimum_speed, goc_maximum_speed, goc_maximum_depth;
    double silicate_climatology;
    int32_t open_bottom, reserved0;
} obgc_pisces_params;

/* TwoBandPhotosyntheticallyActiveRadiation parameters (src/Light/2band.jl:106-117). */
typedef struct obgc_twoband_params {
    double water_red_attenuation;
    double water_blue_attenuation;
    double chlorophyll_red_attenuation;
    double chlorophyll_blue_attenuation;
    double chlorophyll_red_exponent;
    double chlorophyll_blue_exponent;
    double pigment_ratio;
    double phytoplankton_chlorophyll_ratio;
} obgc_twoband_params;

/* Surface PAR forms accepted by the light models (src/Light/2band.jl:91-103; Light.jl:45-47). */
enum obgc_surface_par {
    OBGC_SURFACE_PAR_DEFAULT = 0,  /* default_surface_PAR(t) = 100*max(0, cos(t*pi/12h))      */
    OBGC_SURFACE_PAR_CONSTANT = 1, /* `value`                                                   */
    OBGC_SURFACE_PAR_FIELD = 2     /* per-column device array (Nx*Ny, i fastest), same dtype as the grid fields */
};
typedef struct obgc_surface {
    int32_t kind;                  /* enum obgc_surface_par                                     */
    int32_t reserved0;
    double value;                  /* OBGC_SURFACE_PAR_CONSTANT                                 */
    const void* field;             /* OBGC_SURFACE_PAR_FIELD (device)                           */
} obgc_surface;

/* Grid topologies (Oceananigans RectilinearGrid). z is always Bounded. */
enum obgc_topology { OBGC_PERIODIC = 0, OBGC_BOUNDED = 1, OBGC_FLAT = 2 };

/*
 * A rectilinear grid with uniform spacing and the Oceananigans field layout: column-major,
 * i fastest, k = 0 at the bottom, k = Nz-1 at the surface.  Strides are in elements; stride_i is
 * 1.  An Oceananigans OffsetArray with halos is described by pointing at its first interior
 * element and passing stride_j = Nx+2Hx, stride_k = (Nx+2Hx)(Ny+2Hy); the engine never reads or
 * writes halo cells (periodic neighbours are wrapped in-kernel).
 */
typedef struct obgc_grid {
    int32_t Nx, Ny, Nz;
    int32_t topology_x, topology_y;   /* enum obgc_topology */
    int32_t reserved0;
    double Lx, Ly, Lz;                /* extents (m); z faces at -Lz + k*Lz/Nz                */
    int64_t stride_j, stride_k;
} obgc_grid;

/* ---------------------------------------------------------------------------------------
 * Library info
 * ------------------------------------------------------------------------------------- */
int obgc_abi_version(void);
/* Human-readable text of the last error raised on the calling host thread. */
const char* obgc_last_error_message(void);
/* Number of kernels this library has launched in this process (all entry points). */
int64_t obgc_kernel_launch_count(void);
/* Measured FP64 FMA rate of the device (GFLOP/s, 2 per FMA): the denominator of the FP64
 * kernels' rooflines.  Runs a few 10-ms probe launches on `stream` and synchronises it. */
int obgc_fp64_fma_peak(double* gflops, void* stream);

/* ---------------------------------------------------------------------------------------
 * NutrientsPlanktonDetritus model description (host only, no device work)
 * ------------------------------------------------------------------------------------- */

/* Fill `out` with the LOBSTER (constructors.jl:65-96) or NPZD (constructors.jl:177-227)
 * defaults.  LOBSTER: NitrateAmmonia, PhytoZoo, TwoParticleAndDissolved; NPZD: Nutrient, PhytoZoo
 * with Q10 = 1.88, linear P mortality, analytical light limitation, single-class Detritus. */
int obgc_npd_preset(int32_t preset, obgc_npd_params* out);

/* required_biogeochemical_tracers (NutrientsPlanktonDetritus.jl:69-74): writes the names
 * (enum obgc_tracer) in the reference's order into names[0..cap) and returns the count (<0 on
 * error). */
int obgc_npd_required_tracers(const obgc_npd_params* p, int32_t* names, int32_t cap);

/* biogeochemical_drift_velocity (plankton.jl:60-63, detritus.jl:135-141,290-291): writes the
 * w-component of tracer `name`'s drift velocity on the Nz+1 z-faces (m/s, bottom first) of a grid
 * with Nz levels, exactly as setup_velocity_fields builds it.  Returns 1 if the tracer drifts, 0 if
 * not (w_faces left untouched), <0 on error. */
int obgc_npd_drift_velocity(const obgc_npd_params* p, int32_t name, int32_t Nz, double* w_faces);

/* conserved_tracers(bgc) (NutrientsPlanktonDetritus/coupling_utils.jl:1-52): group 0 is the
 * nitrogen tracers (scale factors 1), group 1 the carbon tracers with their scale factors (only with
 * the carbonate system).  Returns the member count, or <0 when the group does not exist. */
int obgc_npd_conserved_tracers(const obgc_npd_params* p, int32_t group, int32_t* names, double* scalefactors,
                               int32_t cap);

/* ScaleNegativeTracers(tracers; scalefactors, invalid_fill_value) applied once to n_fields (<= 8)
 * fields on the grid's interior (update_biogeochemical_state!(model, ::ScaleNegativeTracers),
 * src/Utils/negative_tracers.jl:136-276).  scalefactors NULL = ones. */
int obgc_scale_negatives(const obgc_grid* grid, int32_t dtype, int32_t n_fields, void* const* fields,
                         const double* scalefactors, double invalid_fill_value, void* stream);
/* ZeroNegativeTracers applied once: max(0, c) on each of n_fields (<= 16) fields
 * (src/Utils/negative_tracers.jl:23-29). */
int obgc_zero_negatives(const obgc_grid* grid, int32_t dtype, int32_t n_fields, void* const* fields, void* stream);

/* Continuous-form functor (bgc)(Val(:X), x, y, z, t, tracers..., PAR) for one point, host side
 * (docs/src/model_implementation.md:75, src/BoxModel/timesteppers.jl:60-61).  `values` holds
 * OBGC_NUM_NAMED entries indexed by enum obgc_tracer (absent tracers ignored).  Writes the
 * tendency of `name` to *out. */
int obgc_npd_eval_point(const obgc_npd_params* p, int32_t name, double x, double y, double z,
                        double t, const double* values, double PAR, double* out);

/* ---------------------------------------------------------------------------------------
 * Stateless device kernels (functional entry points)
 * ------------------------------------------------------------------------------------- */

/* Discrete-form tendencies of every BGC tracer at every cell (mode (i) of the drop-in): replaces
 * the per-tracer functor calls (bgc)(i, j, k, grid, Val(:X), clock, fields, auxiliary_fields)
 * (NutrientsPlanktonDetritus.jl:88; src/OceanBioME.jl:158-159) that Oceananigans inlines into one
 * tendency kernel per tracer.  fields[name] / G[name]: device pointers (NULL where absent), all of
 * dtype `dtype` on `grid`'s layout; PAR: device field of the same layout. */
int obgc_npd_tendencies(const obgc_npd_params* p, const obgc_grid* grid, int32_t dtype,
                        const void* const* fields, const void* PAR, void* const* G,
                        double t, void* stream);

/* TwoBand PAR (update_TwoBandPhotosyntheticallyActiveRadiation!, src/Light/2band.jl:1-33 and
 * its update, :148-155): PAR from phytoplankton P, one column scan per (i, j). */
int obgc_twoband_par(const obgc_twoband_params* lp, const obgc_surface* surface,
                     const obgc_grid* grid, int32_t dtype, const void* P, void* PAR,
                     double t, void* stream);

/* MultiBand PAR (update_MultiBandPhotosyntheticallyActiveRadiation!, src/Light/multi_band.jl:
 * 147-185) for `nbands` bands: band_fields[n] written per band and PAR_total = sum of bands.
 * kw, e, chi, division: nbands host doubles (the band-mean coefficients of multi_band.jl:93-104 and
 * surface_PAR_division).  Chl: device chlorophyll field (mg Chl/m3). */
int obgc_multiband_par(int32_t nbands, const double* kw, const double* e, const double* chi,
                       const double* division, const obgc_surface* surface,
                       const obgc_grid* grid, int32_t dtype, const void* Chl,
                       void* const* band_fields, void* PAR_total, double t, void* stream);

/* Band means of Morel (1988) coefficients (numerical_mean, multi_band.jl:93-104,136-140), host. */
int obgc_multiband_coefficients(int32_t nbands, const double* band_edges /* 2*nbands nm */,
                                int32_t nbase, const double* base_lambda, const double* base_kw,
                                const double* base_e, const double* base_chi,
                                double* kw, double* e, double* chi);

/* Euphotic depth (_compute_euphotic_depth!, src/Light/compute_euphotic_depth.jl:3-29): first
 * depth where PAR <= cutoff * surface PAR, log-interpolated; writes Nx*Ny values.  The surface
 * value (PAR[Nz] + PAR[Nz+1])/2 of the reference is the surface PAR of a field whose top halo holds
 * the value-boundary-condition mirror, so it is taken from `surface` at time t.  Columns that never
 * cross the cutoff get the centre of the cell below the bottom. */
int obgc_euphotic_depth(const obgc_surface* surface, const obgc_grid* grid, int32_t dtype,
                        const void* PAR, void* zeu, double cutoff, double t, void* stream);

/* ---------------------------------------------------------------------------------------
 * Carbon chemistry (src/Models/CarbonChemistry)
 * ------------------------------------------------------------------------------------- */
enum obgc_carbon_output {
    OBGC_OUT_FCO2 = 0,   /* selected_output Val(:fCO₂) (carbon_chemistry.jl:167)  */
    OBGC_OUT_PCO2 = 1,   /* Val(:pCO₂) (:170-193)                                  */
    OBGC_OUT_PH_FREE = 2,/* Val(:pHᶠ) (:168)                                      */
    OBGC_OUT_PH_TOTAL = 3,/* Val(:pHᵗ) (:195-200)                                 */
    OBGC_OUT_PH_SWS = 4, /* Val(:pHˢ) (:202-210)                                   */
    OBGC_OUT_H = 5,      /* the solved free [H+] (mol/kg)                          */
    OBGC_OUT_CARBONATE = 6,/* carbonate_concentration (calcite_concentration.jl:1-53) */
    OBGC_OUT_OMEGA_CALCITE = 7 /* calcite_saturation (calcite_concentration.jl:55-80)  */
};
/* Seawater density of the unit conversions: the reference's default teos10_polynomial_approximation
 * (src/Models/seawater_density.jl:33-39, the Roquet et al. 2015 TEOS-10 polynomial fed as the
 * reference feeds it), UNESCO EOS-80, or a constant. */
enum obgc_density { OBGC_DENSITY_EOS80 = 0, OBGC_DENSITY_CONSTANT = 1, OBGC_DENSITY_TEOS10_POLYNOMIAL = 2 };

/*
 * Options of a batched carbonate solve, mirroring the keyword arguments of
 * (p::CarbonChemistry)(; DIC, T, S, Alk, pH, P, output, boron, sulfate, fluoride, silicate,
 * phosphate, initial_pH_guess) (carbon_chemistry.jl:111-121) and the DampedNewtonRaphsonSolver
 * defaults (src/Utils/solvers.jl:81-88, carbon_chemistry.jl:81).
 */
typedef struct obgc_carbon_options {
    int32_t output;              /* enum obgc_carbon_output                                   */
    int32_t density;             /* enum obgc_density                                         */
    int32_t has_pressure;        /* 0: P = nothing (no pressure correction); 1: use P          */
    int32_t ph_given;            /* 1: `pH` array supplies free pH, no solve                  */
    int32_t max_iters;           /* Newton iterations (reference default 100)                 */
    int32_t warm_start;          /* 1: start from H_inout instead of 10^-initial_pH_guess     */
    double density_value;        /* OBGC_DENSITY_CONSTANT                                     */
    double initial_pH_guess;     /* 8                                                        */
    double atol;                 /* 1e-20                                                     */
    double damping;              /* 0.5                                                       */
    double armijo_constant;      /* 0.5                                                       */
    double min_damping;          /* 0.5^10                                                    */
    double calcium_ion_per_salinity; /* 0.0103/35 (calcite_concentration.jl:78)             */
    int32_t saturation_mineral;  /* Omega's solubility product (the CarbonChemistry's
                                  * calcite_solubility): 0 KSP_calcite, 1 KSP_aragonite
                                  * (equilibrium_constants.jl:740-850)                         */
    int32_t reserved0;
} obgc_carbon_options;

int obgc_carbon_default_options(obgc_carbon_options* out);

/* ---------------------------------------------------------------------------------------
 * Air-sea gas exchange (src/Models/GasExchange): the flux k (C_water - C_air) through the
 * surface face of each column, positive out of the ocean (Oceananigans' top FluxBoundaryCondition,
 * GasExchange functor gas_exchange.jl:26-39).
 *   k = k660(u10) / sqrt(Sc(T) / 660) * solubility(T, S)       (gas_transfer_velocity.jl:30-31)
 *   CO2: C_water = pCO2 of the surface cell's DIC, Alk, T, S (CarbonChemistry, FP64 solve;
 *        carbon_dioxide_concentration.jl:48-60), C_air in ppmv, solubility = K0(T, S) rho(T, S) / 1000
 *        (gas_solubility.jl:62-64), flux in mmol C / m2 / s
 *   O2:  C_water = the surface O2, C_air = air_concentration * beta(T, S) / Tk (Wanninkhof 1992,
 *        gas_solubility.jl:38-56, evaluated as written there), solubility = 1
 * ------------------------------------------------------------------------------------- */
enum obgc_gas { OBGC_GAS_CO2 = 0, OBGC_GAS_O2 = 1 };

typedef struct obgc_gas_exchange {
    int32_t gas;                 /* enum obgc_gas                                              */
    int32_t reserved0;
    double k660[4];              /* k660(u) = k660[0] + k660[1] u + k660[2] u^2 + k660[3] u^3
                                  * (m/s); default Ho06: (0, 0, 0.266 / 3600 / 100, 0)         */
    double schmidt[5];           /* Sc(T) = s0 + s1 T + s2 T^2 + s3 T^3 + s4 T^4, T in degC       */
    double wind_speed;           /* u10 (m/s) when wind_field is NULL (default 2)              */
    const void* wind_field;      /* (Nx, Ny) dense, grid dtype, or NULL                        */
    double air_concentration;    /* CO2: ppmv (413); O2: mmol/m3 (9352.7)                      */
    const void* air_field;       /* (Nx, Ny) dense, grid dtype, or NULL                        */
    double o2_solubility[6];     /* A1 A2 A3 B1 B2 B3 (OxygenSolubility defaults)              */
    obgc_carbon_options carbon;  /* the pCO2 solve (output is set to pCO2)                     */
} obgc_gas_exchange;

/* CarbonDioxideGasExchangeBoundaryCondition() / OxygenGasExchangeBoundaryCondition() defaults
 * (GasExchange.jl:96-146, schmidt_number.jl, gas_transfer_velocity.jl:53-59). */
int obgc_gas_exchange_defaults(int32_t gas, obgc_gas_exchange* out);
/* Flux of every column (Nx, Ny dense, FP64 out) from the surface cells (k = Nz-1) of the 3-D
 * fields T, S and DIC, Alk (CO2) or O2 (O2; the others may be NULL), of dtype `dtype`. */
int obgc_gas_exchange_flux(const obgc_gas_exchange* g, const obgc_grid* grid, int32_t dtype, const void* T,
                           const void* S, const void* DIC, const void* Alk, const void* O2, double* flux,
                           void* stream);
/* One column on the host (the same device function), e.g. for a BoxModel-style driver. */
int obgc_gas_exchange_point(const obgc_gas_exchange* g, double T, double S, double DIC, double Alk, double O2,
                            double u10, double air, double* flux);

/*
 * Batched FP64 carbonate solve on the device: n cells.  Inputs DIC (mmol/m3), Alk (meq/m3),
 * T (degC), S (psu) of dtype `dtype`; optional (NULL = zero / absent) silicate, phosphate
 * (mmol/m3), P (bar), pH (free pH, when ph_given).  H_inout (FP64, optional) receives the solved
 * [H+] and, with warm_start, supplies the start.  out: FP64 array of n.  iters (optional int32 n):
 * Newton iterations used.  Returns OBGC_ERR_NOT_CONVERGED if any cell hit max_iters with
 * |residual| > atol (all outputs still written).
 */
int obgc_carbon_chemistry(const obgc_carbon_options* opt, int64_t n, int32_t dtype,
                          const void* DIC, const void* Alk, const void* T, const void* S,
                          const void* silicate, const void* phosphate, const void* P,
                          const void* pH, double* H_inout, double* out, int32_t* iters,
                          void* stream);

/* Host (CPU) evaluation of the same functor for one point, FP64 (used by the Julia shim for
 * diagnostics and by the continuous-form path). */
int obgc_carbon_chemistry_point(const obgc_carbon_options* opt, double DIC, double Alk,
                                double T, double S, double silicate, double phosphate,
                                double P, double pH, double* out);

/* ---------------------------------------------------------------------------------------
 * 3-D model context: fused advection + BGC + RK3 (mode (ii)) and the plugin hooks (mode (i))
 * ------------------------------------------------------------------------------------- */
typedef struct obgc_ctx obgc_ctx;

enum obgc_advection { OBGC_ADVECTION_NONE = 0, OBGC_ADVECTION_WENO5 = 1 };

typedef struct obgc_model_desc {
    obgc_npd_params npd;          /* the biogeochemistry                                      */
    obgc_twoband_params light;    /* TwoBand light attenuation                                */
    obgc_surface surface;         /* surface PAR                                              */
    obgc_grid grid;
    int32_t precision;            /* enum obgc_precision                                      */
    int32_t advection;            /* enum obgc_advection (tracer + drift advection scheme)    */
    int32_t n_passive;            /* extra advected tracers (obgc_fields.passive[0..n_passive)):
                                     zero BGC tendency unless passive_tendency_of says otherwise */
    int32_t carry_T;              /* T carried as an advected tracer even if BGC ignores it   */
    int32_t carry_S;              /* S carried as an advected tracer                          */
    int32_t negatives;            /* enum obgc_negatives                                      */
    uint32_t zero_exclude;        /* ZeroNegativeTracers exclude: bit n = enum obgc_tracer n,
                                     bit 21 + p = passive tracer p                            */
    int32_t reserved1;
    double invalid_fill_value;    /* ScaleNegativeTracers(...; invalid_fill_value) (NaN)      */
    /* CarbonateSystem(N) replicates (carbonate_system.jl:41-83): passive tracer p takes the BGC
     * tendency of tracer passive_tendency_of[p] - 1 (OBGC_DIC or OBGC_ALK; 0: none), as DIC2..DICN
     * and Alk2..AlkN evaluate the DIC and Alk functors.  DIC1 / Alk1 are the named DIC / Alk. */
    int8_t passive_tendency_of[OBGC_MAX_PASSIVE];
} obgc_model_desc;

/* Fields a context works on.  Tracer arrays are device pointers of the context's state dtype
 * (FP32 for OBGC_PREC_F32, FP64 otherwise); velocities u, v (Face, Center, Center / Center, Face,
 * Center) and w (Center, Center, Face: w[k] on the face below cell k) are the same dtype and
 * layout, or NULL for zero.  G (mode (i)) receives BGC tendencies; PAR is written by
 * obgc_update_state.  All pointers may be re-bound at any time. */
typedef struct obgc_fields {
    void* tracers[OBGC_NUM_NAMED];
    void* passive[OBGC_MAX_PASSIVE];
    const void* u;
    const void* v;
    const void* w;
    void* PAR;
    void* G[OBGC_NUM_NAMED];
} obgc_fields;

/* Build a context (src/OceanBioME.jl:100-120 Biogeochemistry(...); Oceananigans
 * NonhydrostaticModel(grid; biogeochemistry, advection)).  Allocates the RK3 tendency and
 * ping-pong buffers on the current device. */
int obgc_create(const obgc_model_desc* desc, obgc_ctx** out);
int obgc_destroy(obgc_ctx* ctx);
/* Bind (or re-bind) device fields. */
int obgc_bind_fields(obgc_ctx* ctx, const obgc_fields* fields);
/* update_biogeochemical_state! (src/OceanBioME.jl:161-167; 2band.jl:148-155): PAR at time t. */
int obgc_update_state(obgc_ctx* ctx, double t, void* stream);
/* Mode (i): BGC tendencies of all tracers into fields.G at time t (uses the bound PAR). */
int obgc_compute_tendencies(obgc_ctx* ctx, double t, void* stream);
/* Mode (ii): nsteps fused RK3 steps of size dt from time t (Oceananigans time_step! with
 * RungeKutta3: per substep PAR scan + fused WENO5/drift/BGC/RK3 update).  The bound tracer arrays
 * hold the state before and after. */
int obgc_step(obgc_ctx* ctx, double t, double dt, int32_t nsteps, void* stream);
/* Capture `nsteps` steps into a CUDA graph owned by the context and replay it (same semantics as
 * obgc_step; re-captured when dt, nsteps or bindings change). */
int obgc_step_graph(obgc_ctx* ctx, double t, double dt, int32_t nsteps, void* stream);
/* Device-side status of the fused step.  Every obgc_step / obgc_step_graph call clears a per-context
 * device word, and its kernels set flags in it: OBGC_FLAG_NAN when a substep writes a NaN or an
 * infinity into the state (the reference lets NaN propagate, src/Utils/negative_tracers.jl:197,266;
 * Oceananigans' NaNChecker stops a simulation on one), OBGC_FLAG_NOT_CONVERGED when a surface pCO2
 * solve of the gas exchange ends unconverged (src/Utils/solvers.jl:118 warns).  The word is copied
 * to pinned host memory behind the call's last kernel.
 *   obgc_step_status waits for the context's last call and returns OBGC_ERR_NAN (NaN first) or
 *   OBGC_ERR_NOT_CONVERGED when a flag is set, else OBGC_OK; flags (optional) receives the word.
 *   obgc_set_status_check(ctx, 1) (the default) makes obgc_step itself wait for its kernels and
 *   return that status; with 0, obgc_step returns as soon as the work is enqueued.  obgc_step_graph
 *   never waits: call obgc_step_status after it.
 * OBGC_FLAG_TIMEOUT (status OBGC_ERR_TIMEOUT) reports a tile copy of the tensor-memory accelerator
 * that a block stopped waiting for after a bounded number of polls. */
enum obgc_step_flags { OBGC_FLAG_NAN = 1, OBGC_FLAG_NOT_CONVERGED = 2, OBGC_FLAG_TIMEOUT = 4 };
int obgc_step_status(obgc_ctx* ctx, int32_t* flags);
int obgc_set_status_check(obgc_ctx* ctx, int32_t on);
/* One RK3 stage (0, 1 or 2) of the step that starts at time t (Oceananigans rk3_substep! followed
 * by update_state!, as inside obgc_step), from the caller's arrays in[] into out[] (one per slot in
 * the context's order: the model's tracers, then passive tracers; the bound grid's layout and
 * strides; in[q] != out[q]).  The context keeps the previous stage's tendencies, so the three
 * stages of a step run in order on one context.  The entering state is taken as it is (obgc_step
 * runs the negative-tracer modifier once on its entering state; here the caller's state is
 * already past update_state!).  This is the form a domain split across GPUs needs: a y slab with
 * three halo rows on each side (a Periodic-y grid of Ny_slab + 6 rows) exchanges its halos between
 * stages (obgc_halo_pack / obgc_halo_unpack), as Oceananigans' distributed architecture fills
 * halos before each tendency computation.  Status as obgc_step (the status word is cleared by
 * stage 0 and collects the step's three stages). */
int obgc_substep(obgc_ctx* ctx, double t, double dt, int32_t stage, const void* const* in, void* const* out,
                 void* stream);
/* Halo rows of a y slab.  `slab` is the slab's grid: Ny = Ny_slab + 2 * halo rows, rows [halo,
 * Ny - halo) its own.  pack copies the slab's first `halo` own rows (those its southern neighbour
 * needs) into `south` and its last `halo` own rows into `north`; unpack writes `south` (the
 * southern neighbour's `north` buffer) into rows [0, halo) and `north` (the northern neighbour's
 * `south` buffer) into rows [Ny - halo, Ny).  Buffers: dense [n_fields][Nz][halo][Nx] of dtype.
 * n_fields <= 32.  No counterpart in the reference (Oceananigans' fill_halo_regions! over MPI
 * plays this part); the exchange of the buffers between ranks is the caller's (NCCL send/recv). */
int obgc_halo_pack(const obgc_grid* slab, int32_t dtype, int32_t n_fields, const void* const* fields, int32_t halo,
                   void* south, void* north, void* stream);
int obgc_halo_unpack(const obgc_grid* slab, int32_t dtype, int32_t n_fields, void* const* fields, int32_t halo,
                     const void* south, const void* north, void* stream);
/* Device kernel time of the last obgc_step / obgc_step_graph measured with CUDA events on the
 * launching stream (ms); with profiling on, also the summed duration of the fused substep kernel
 * launches (event pairs around each launch).  launches: kernels the call enqueued. */
int obgc_last_step_timing(const obgc_ctx* ctx, double* total_ms, double* substep_ms,
                          int64_t* launches);
/* How the fused substep stages its tiles.  mode 1 (the default): with the tensor-memory
 * accelerator when the steps qualify (FP32 arithmetic: OBGC_PREC_F32 or OBGC_PREC_MIXED; no
 * passive tracers, no model w, and none of the optional terms: closure, gas exchange, forcing,
 * fused modifier, sediment, replicates); a call then copies the bound arrays into a padded context
 * copy with their periodic images, runs its stages through two padded copies and writes the bound
 * arrays in its last stage, every stage copying each tracer's tile of a level with one tensor copy
 * (no copy when no tile needs the periodic wrap: the first stage reads the bound arrays through
 * tensor maps).  OBGC_PREC_MIXED: the padded copies hold the FP64 state rounded to FP32 (the copy
 * rounds it, every stage but the last writes the next one) and every stage updates the FP64 bound
 * arrays in place; a model with a sinking tracer outside the two flux pre-pass slots, or with
 * segments whose chlorophyll sums the pre-pass does not form (obgc_set_tiling(1)), keeps cp.async.
 * mode 0: per-element cp.async staging always.  obgc_get_staging reports whether the context has the padded copies and tensor
 * maps (available) and whether the last obgc_step / obgc_step_graph capture used them. */
int obgc_set_staging(obgc_ctx* ctx, int32_t mode);
int obgc_get_staging(const obgc_ctx* ctx, int32_t* available, int32_t* last_used);
/* Bracket every fused substep launch of obgc_step with CUDA events (off by default). */
int obgc_set_profiling(obgc_ctx* ctx, int32_t on);
/* Vertical segment length (levels) of the fused kernel's work items (default: chosen per grid, 8 when the grid has enough tiles to fill the GPU, down to 2). */
int obgc_set_tiling(obgc_ctx* ctx, int32_t levels_per_item);
/* Autotune the fused step's launch shape on the bound state: for each candidate vertical segment
 * length (2 .. 32 levels, capped at Nz) and tile staging (tensor copies where available, and
 * cp.async), one warm-up step and `steps` timed steps of obgc_step(t, dt) from the saved state.
 * Keeps the fastest (obgc_set_tiling / obgc_set_staging) and returns it with its ms per step (any
 * output may be NULL).  The bound tracers, the sediment storages and the gas exchange's [H+] are
 * restored before it returns, so the caller's state is unchanged; synchronizes the stream.
 * The reference's functors (src/OceanBioME.jl:157-159) run inside Oceananigans' tendency kernels,
 * launched with a fixed workgroup shape and no tuner. */
int obgc_autotune_step(obgc_ctx* ctx, double t, double dt, int32_t steps, int32_t* levels_per_item,
                       int32_t* staging, double* ms_per_step, void* stream);
/* Air-sea gas exchange as the top boundary condition of the fused step (obgc_step, obgc_step_graph):
 * FieldBoundaryConditions(top = CarbonDioxideGasExchangeBoundaryCondition()) on DIC (g->gas CO2;
 * the model carries DIC, Alk, T and S) or OxygenGasExchangeBoundaryCondition() on O2 (the model
 * carries O2, T and S).  Each RK3 stage computes the flux of every column from the stage's surface
 * cells and the surface cell's tendency loses flux / dz.  g = NULL with `gas` clears that gas. */
int obgc_set_gas_exchange(obgc_ctx* ctx, int32_t gas, const obgc_gas_exchange* g);
/* The same condition on any tracer (a code of OBGC_PASSIVE's form): g->gas CO2 with the water's
 * CO2 from the tracers `dic` and `alk` (CarbonDioxideConcentration(; DIC = :DIC2, Alk = :Alk2),
 * carbon_dioxide_concentration.jl:13-60), or O2 with the tracer itself as the water's O2.  Up to
 * OBGC_MAX_GAS_CONDITIONS conditions, one per tracer; g = NULL removes the tracer's condition.
 * obgc_set_gas_exchange(ctx, CO2, g) is obgc_set_gas_exchange_on(ctx, OBGC_DIC, g, OBGC_DIC, OBGC_ALK). */
#define OBGC_MAX_GAS_CONDITIONS 4
int obgc_set_gas_exchange_on(obgc_ctx* ctx, int32_t tracer, const obgc_gas_exchange* g, int32_t dic, int32_t alk);
/* forcing = (; X = F): a prescribed source rate (tracer units per second) added to tracer X's
 * tendency in the fused step at every RK3 stage whose time t (Oceananigans' stage clock) satisfies
 * t_start <= t < t_end (+-INFINITY for always).  `rate` is a device field of the context's state
 * dtype on the grid's layout; it stays the caller's and is read at every stage.  With a spatial
 * mask it expresses the windowed release of examples/oae_experiment.jl:55-79.  Up to
 * OBGC_MAX_FORCINGS tracers; rate = NULL removes the tracer's forcing. */
#define OBGC_MAX_FORCINGS 4
int obgc_set_forcing(obgc_ctx* ctx, int32_t tracer, const void* rate, double t_start, double t_end);
/* closure = ScalarDiffusivity(κ) (explicit time discretization) on every tracer of the fused step:
 * a horizontal diffusivity kappa_h (m2/s, x and y faces) and a vertical one, kappa_z constant or
 * kappa_z_faces[Nz + 1] (face f below cell f; the bottom and top faces are walls and carry no
 * flux), added to the advective face fluxes (VerticalScalarDiffusivity: kappa_h = 0;
 * HorizontalScalarDiffusivity: kappa_z = 0).  Zero everywhere switches it off. */
int obgc_set_diffusivity(obgc_ctx* ctx, double kappa_h, double kappa_z, const double* kappa_z_faces);
/* The vertical part's time discretization: OBGC_EXPLICIT (default) or OBGC_VERTICALLY_IMPLICIT
 * (VerticalScalarDiffusivity(VerticallyImplicitTimeDiscretization(), κ)): after each RK3 stage's
 * explicit update U* (advection, BGC, horizontal diffusion), every column of every tracer solves
 * (I - dt_s d/dz kappa d/dz) U = U* with dt_s = (gamma + zeta) dt and no flux through the bottom
 * and top faces, then the negative-tracer modifier runs. */
enum obgc_time_discretization { OBGC_EXPLICIT = 0, OBGC_VERTICALLY_IMPLICIT = 1 };
int obgc_set_vertical_time_discretization(obgc_ctx* ctx, int32_t discretization);
/* sediment = InstantRemineralisationSediment(grid; sinking_tracers, remineralisation_reciever,
 * burial_efficiency_constant1 = a (0.013), _constant2 = b (0.53), _half_saturation = k (7/6.56))
 * (src/Models/Sediments/instant_remineralisation.jl): per RK3 stage the sinking fluxes of the
 * named tracers (enum obgc_tracer) through the bottom face deposit F per column, e = a + b (F/(k+F))^2
 * of it is buried in the column's storage (stepped with the same RK3 stages) and (1 - e) F / dz is
 * returned to the receiver's bottom cell.  n_sinking = 0 removes it. */
int obgc_set_sediment(obgc_ctx* ctx, int32_t n_sinking, const int32_t* sinking_names, int32_t receiver_name,
                      double a, double b, double k);
/* The sediment storage of every column (Ny x Nx dense, FP64 on the host): `set` (optional) replaces
 * it, then `get` (optional) receives it.  Synchronises the device. */
int obgc_sediment_storage(obgc_ctx* ctx, const double* set, double* get);

/* sediment = SimpleMultiGSediment(grid; ...) (src/Models/Sediments/simple_multi_G.jl:15-430; the
 * nitrogen-only form, sinking_carbon = nothing): a single-layer sediment per column with slow, fast
 * and refractory organic nitrogen (Ns, Nf, Nr, mmol N/m2), fed by the sinking fluxes of the named
 * tracers through the bottom face and returning its remineralisation to the bottom cell's NH4 and
 * NO3 and drawing O2 (Soetaert et al. 2000 fractions: ammonia oxidation, denitrification, anoxic
 * remineralisation, solid deposition).  It is coupled as BiogeochemicalSediment does
 * (src/Sediments/update_state.jl:6-17, tracer_coupling.jl, tracked_fields.jl): after every RK3 stage
 * of the water, the bottom-cell NO3, NH4, O2 and the sinking fluxes are tracked from the new state,
 * the sediment takes a full RK3 step (timesteppers.jl:48-73) of the stage's length ((gamma + zeta)
 * dt), its first stage from the tendency cached at the end of its previous step, and the coupled
 * tendencies (sediment_tendency / dz) enter the bottom cells of the next water stage.  The model
 * needs NO3, NH4 and O2 (LOBSTER with Oxygen).  n_sinking = 0 removes it. */
typedef struct obgc_multig_params {
    double fast_decay_rate;          /* 2 / day                                              */
    double slow_decay_rate;          /* 0.2 / day                                            */
    double fast_redfield;            /* 0.1509 (the carbon form's)                           */
    double slow_redfield;            /* 0.13                                                 */
    double fast_fraction;            /* 0.74                                                 */
    double slow_fraction;            /* 0.26                                                 */
    double refactory_fraction;       /* 0.1                                                  */
    double sedimentation_rate;       /* cm/year; <= 0: 982 |z_bottom|^-1.548 of the grid      */
    double anoxia_half_saturation;   /* 1 mmol/m3                                            */
    double sinking_redfield;         /* 6.56: C:N of the sinking nitrogen                     */
    double nitrate_oxidation[6];     /* A..F of the ammonia oxidation fraction's fit          */
    double denitrification[6];
    double anoxic[6];
} obgc_multig_params;
/* The reference's SimpleMultiGSediment keyword defaults (sedimentation_rate left <= 0: from the grid). */
int obgc_multig_default_params(obgc_multig_params* p);
int obgc_set_multig_sediment(obgc_ctx* ctx, const obgc_multig_params* p, int32_t n_sinking, const int32_t* sinking_names);
/* The sediment's fields [3][Ny][Nx] (Ns, Nf, Nr; FP64 on the host): `set` (optional) replaces them
 * (and restarts its clock: the next step computes its first tendency afresh), then `get` (optional)
 * receives them.  Synchronises the device. */
int obgc_multig_sediment_state(obgc_ctx* ctx, const double* set, double* get);
/* Size and selected field offsets of the ABI structs (which: 0 npd_params, 1 twoband,
 * 2 surface, 3 grid, 4 carbon_options, 5 model_desc, 6 fields, 7 column_spec, 8 columns_desc,
 * 9 pisces_params, 10 pisces_phyto, 11 pisces_field, 12 gas_exchange, 13 box_drivers) for binding
 * self-checks; no counterpart in the reference. */
int obgc_struct_layout(int32_t which, int64_t* out, int32_t cap);

/* Domain-integrated mass of a conserved group (conserved_tracers, NutrientsPlanktonDetritus/
 * coupling_utils.jl:1-52): sum over cells of sum_n scale[n]*tracer_n, accumulated in FP64 with
 * compensated summation.  group: 0 nitrogen, 1 carbon.  Result written to *total (host). */
int obgc_tracer_budget(obgc_ctx* ctx, int32_t group, double* total, void* stream);

/*
 * The same compensated FP64 budget reduction as obgc_tracer_budget, for callers that cannot
 * allocate device memory.  No counterpart in the reference.
 *
 * Who needs it: a host whose device memory is owned by another allocator (CUDA.jl's or PyTorch's
 * caching pool, where a foreign cudaMalloc fragments the pool or exceeds its reservation), and
 * callers that run under a fixed device-memory budget (the column service admits runs against
 * one).  Such callers cannot create a context, whose set-up allocates its reduction buffer.
 *
 * This entry point allocates nothing: its partial sums live in a file-scope device array of
 * OBGC_BUDGET_STATIC_SLOTS entries (16 bytes each, 16 KiB in total), which every GPU that loads the
 * library holds until the process exits.  fields[0..n_fields) are device arrays of dtype `dtype`
 * on `grid`'s layout, scale[0..n_fields) host doubles; the result sum over cells of
 * sum_n scale[n]*fields[n] is written to *total (host) and the call returns after the stream has
 * finished it.  n_fields above OBGC_BUDGET_STATIC_MAX_FIELDS is rejected (OBGC_ERR_INVALID_ARGUMENT).
 *
 * The call synchronizes `stream` (the sum comes back to the host), so no call of it can be
 * captured into a CUDA graph.  The first call on each device looks up the array's device address
 * on that device.  The address is kept for the life of the process: after
 * a cudaDeviceReset (or any teardown of the device's primary context) the library's module is
 * loaded again elsewhere, so do not call this entry point on that device again.  All calls share
 * the one array: calls that overlap on the GPU (different streams or host threads without
 * ordering) race and corrupt each other's sums.
 */
#define OBGC_BUDGET_STATIC_SLOTS 1024
#define OBGC_BUDGET_STATIC_MAX_FIELDS 8
int obgc_tracer_budget_static(const obgc_grid* grid, int32_t dtype, int32_t n_fields, const void* const* fields,
                              const double* scale, double* total, void* stream);

/* ---------------------------------------------------------------------------------------
 * Batched box models (src/BoxModel): many independent 0-D NutrientsPlanktonDetritus models
 * ------------------------------------------------------------------------------------- */
/*
 * Advance n_models box models nsteps RK3 steps of dt from t0 (BoxModel time_step!,
 * src/BoxModel/timesteppers.jl:30-93).  state: device FP64 array [n_models][OBGC_NUM_NAMED]
 * (row per model, enum obgc_tracer columns) updated in place.  PAR: device FP64
 * [3*nsteps][n_models] with the prescribed PAR at every RK3 stage time (t, t+8/15 dt, t+2/3 dt)
 * of every step (stage-major, so a warp reads one coalesced row), or NULL with par_constant used.  params_per_model: optional device array of n_models
 * obgc_npd_params (NULL = `p` for all).  record_every > 0 writes the state every record_every
 * steps into record [n_records][n_models][OBGC_NUM_NAMED] (SpeedyOutput,
 * src/BoxModel/output_writer.jl).  precision: OBGC_PREC_F64 or OBGC_PREC_F32 (state and math).
 */
int obgc_box_run(const obgc_npd_params* p, const obgc_npd_params* params_per_model,
                 int64_t n_models, double* state, const double* PAR, double par_constant,
                 double t0, double dt, int32_t nsteps, int32_t record_every, double* record,
                 int32_t precision, void* stream);

/* Time-dependent drivers of obgc_box_run_drivers: BoxModel(; forcing, prescribed_tracers)
 * (src/BoxModel/boxmodel.jl:65-87, timesteppers.jl:37-63), sampled at the RK3 stage times like PAR.
 *   prescribed_tracers = (; X = f(t)): before the tendencies of stage s of step n the tracer takes
 *     prescribed[q][(3n + s) * n_models + m] (update_state!), and after step n the value of row
 *     3(n + 1), so a device array of (3 nsteps + 1) rows of n_models.
 *   forcing = (; X = F): F's rate at the stage time, forcing[q][(3n + s) * n_models + m], is added
 *     to X's tendency; 3 nsteps rows.  Forcings that read the model's fields are outside this form. */
#define OBGC_BOX_MAX_DRIVERS 4
typedef struct obgc_box_drivers {
    const double* PAR;           /* as obgc_box_run                                            */
    double par_constant;
    int32_t n_prescribed, n_forced;             /* each <= OBGC_BOX_MAX_DRIVERS              */
    int32_t prescribed_names[OBGC_BOX_MAX_DRIVERS];   /* enum obgc_tracer                     */
    int32_t forced_names[OBGC_BOX_MAX_DRIVERS];
    const double* prescribed[OBGC_BOX_MAX_DRIVERS];   /* device                               */
    const double* forcing[OBGC_BOX_MAX_DRIVERS];      /* device                               */
} obgc_box_drivers;
/* obgc_box_run with prescribed tracers and forcing (drivers->n_prescribed = n_forced = 0 is
 * obgc_box_run). */
int obgc_box_run_drivers(const obgc_npd_params* p, const obgc_npd_params* params_per_model, int64_t n_models,
                         double* state, const obgc_box_drivers* drivers, double t0, double dt, int32_t nsteps,
                         int32_t record_every, double* record, int32_t precision, void* stream);

/* ---------------------------------------------------------------------------------------
 * Batched uneven columns: many independent 1-D water columns (different depth, parameters,
 * step and duration) advanced together.  Each column is the reference's column configuration
 * (examples/column.jl: NonhydrostaticModel on a 1 x 1 x Nz grid with a LOBSTER or NPZD
 * biogeochemistry, TwoBand light, sinking, and a vertical diffusivity treated implicitly as in
 * Oceananigans' VerticallyImplicitTimeDiscretization), RK3 as src/BoxModel/timesteppers.jl:66-93.
 * Columns are packed into thread blocks by cell count and stay in shared memory for a whole
 * launch of up to max_steps steps.
 * ------------------------------------------------------------------------------------- */
/* ---------------------------------------------------------------------------------------------
 * PISCES entry points.
 * ------------------------------------------------------------------------------------------- */
/* Layout of an auxiliary input (PISCES's auxiliary fields are 2-D, 3-D or constant). */
enum obgc_pisces_field_kind {
    OBGC_PF_CONSTANT = 0,   /* `value` everywhere                                               */
    OBGC_PF_XY = 1,         /* (Nx, Ny) field, dense: element i + j*Nx                          */
    OBGC_PF_XYZ = 2,        /* centre field with the grid's strides                              */
    OBGC_PF_ZFACE = 3,      /* z-face field with the grid's strides, Nz+1 levels; the cell uses the
                               mean of its two faces (the ℑz interpolation of the reference)      */
    OBGC_PF_AUTO = 4,       /* sinking velocities only: built from the parameters as the
                               reference's setup does (constant POC speed, depth-dependent GOC
                               from the zmxl and zeu inputs)                                     */
    OBGC_PF_ZPROFILE = 5    /* Nz+1 face values shared by every column; the cell uses the mean of
                               its two faces                                                     */
};
typedef struct obgc_pisces_field {
    int32_t kind;
    int32_t reserved0;
    double value;
    const void* data;            /* device pointer of the call's dtype                           */
} obgc_pisces_field;

/* Default parameters of PISCES(; grid) (PISCES.jl:288-340 and the component constructors). */
int obgc_pisces_default_params(obgc_pisces_params* out);
/* Every PISCES tendency of every interior cell in one pass: the discrete functors
 * (bgc)(i, j, k, grid, Val(name), clock, fields, auxiliary_fields) of all 24 tracers
 * (PISCES.jl:120-123 and the tracer files).  tracers: OBGC_PIS_NUM device fields (T and S
 * included); aux: OBGC_PAUX_NUM inputs; G: OBGC_PIS_NUM_BGC output fields; t: model time (s). */
int obgc_pisces_tendencies(const obgc_pisces_params* p, const obgc_grid* grid, int32_t dtype,
                           const void* const* tracers, const obgc_pisces_field* aux, void* const* G,
                           double t, void* stream);
/* Host FP64 evaluation of one point: values [OBGC_PIS_NUM], aux [OBGC_PAUX_NUM] (sinking velocities
 * already at the centre), z (m), t (s); G [OBGC_PIS_NUM_BGC]. */
int obgc_pisces_eval_point(const obgc_pisces_params* p, const double* values, const double* aux,
                           double z, double t, double* G);
/* compute_mixed_layer_mean! (PISCES/mean_mixed_layer_properties.jl:10-46): the mean of a centre
 * field above the mixed-layer depth, per column; out is an (Nx, Ny) field. */
int obgc_mixed_layer_mean(const obgc_grid* grid, int32_t dtype, const void* field,
                          const obgc_pisces_field* mixed_layer_depth, void* out, void* stream);
/* compute_calcite_saturation! (PISCES/compute_calcite_saturation.jl:9-37): Ω of every cell with
 * P = |z| g 1026 / 1e5 bar and silicate Si (NULL = 0); FP64 solve, output in dtype. */
int obgc_pisces_calcite_saturation(const obgc_carbon_options* opt, const obgc_grid* grid, int32_t dtype,
                                   const void* DIC, const void* Alk, const void* T, const void* S,
                                   const void* Si, void* omega, void* stream);

/* A 3-D PISCES model stepped on the device: every RK3 stage runs update_biogeochemical_state!
 * (PISCES/update_state.jl:1-17 after the MultiBand light of src/Light/multi_band.jl:147-185: PAR
 * bands from PChl + DChl, euphotic depth, mixed-layer PAR, calcite saturation), then all 24
 * tendencies, then one fused kernel for WENO5 advection of the 26 tracers, the sinking of POC, SFe
 * (POC speed) and GOC, BFe, PSi, CaCO3 (GOC speed) and the RK3 update. */
typedef struct obgc_pisces_model obgc_pisces_model;
typedef struct obgc_pisces_model_desc {
    obgc_pisces_params pisces;
    obgc_grid grid;
    int32_t precision;           /* OBGC_PREC_F32, OBGC_PREC_MIXED or OBGC_PREC_F64 (plain FP64) */
    int32_t advection;           /* enum obgc_advection                                        */
    int32_t nbands;              /* MultiBand bands: 3 (PISCES reads PAR₁, PAR₂, PAR₃)           */
    int32_t negatives;           /* OBGC_NEGATIVES_NONE or _SCALE (conserved_tracers(::PISCES)) */
    double kw[4], e[4], chi[4], division[4];   /* band means (obgc_multiband_coefficients)     */
    obgc_surface surface;        /* OBGC_SURFACE_PAR_DEFAULT or _CONSTANT                      */
    double mixed_layer_depth;    /* prescribed, uniform (m, negative)                          */
    double mean_kappa;           /* mean mixed-layer diffusivity (the reference sets 1 when the
                                    model has no closure, PISCES.jl:360-362)                   */
    double invalid_fill_value;
    obgc_carbon_options carbon;
} obgc_pisces_model_desc;

enum obgc_pisces_model_field {
    OBGC_PMF_PAR = 0, OBGC_PMF_PAR1, OBGC_PMF_PAR2, OBGC_PMF_PAR3,   /* centre fields              */
    OBGC_PMF_ZEU = 4, OBGC_PMF_MLPAR = 5,                            /* (Nx, Ny), dense            */
    OBGC_PMF_OMEGA = 6                                               /* centre field               */
};

int obgc_pisces_model_create(const obgc_pisces_model_desc* desc, obgc_pisces_model** out);
int obgc_pisces_model_destroy(obgc_pisces_model* m);
/* tracers: OBGC_PIS_NUM device fields with the grid's strides (state precision: FP32 for
 * OBGC_PREC_F32, FP64 for OBGC_PREC_MIXED and OBGC_PREC_F64); u, v as for obgc_bind_fields, or NULL. */
int obgc_pisces_model_bind(obgc_pisces_model* m, void* const* tracers, const void* u, const void* v);
int obgc_pisces_model_update_state(obgc_pisces_model* m, double t, void* stream);
int obgc_pisces_model_step(obgc_pisces_model* m, double t, double dt, int32_t nsteps, void* stream);
/* One RK3 stage (0, 1, 2) of the step that starts at t, from the 26 tracer arrays `in` into `out`
 * (distinct arrays in the model's grid layout): update_state! on `in`, the functor, the fused
 * substeps; the previous stage's tendencies stay in the model.  finish != 0 applies the
 * negative-tracer modifier to `out` afterwards, as obgc_pisces_model_step does after its last
 * substep.  For a custom stage loop that fills halos between stages (the y-slab split: one
 * NonhydrostaticModel(grid; biogeochemistry = PISCES(...)) per rank of Oceananigans' Distributed
 * architecture, whose fill_halo_regions! runs before each tendency computation). */
int obgc_pisces_model_substep(obgc_pisces_model* m, double t, double dt, int32_t stage, const void* const* in,
                              void* const* out, int32_t finish, void* stream);
/* Device pointer of an auxiliary field the model keeps (state precision). */
int obgc_pisces_model_field(obgc_pisces_model* m, int32_t which, void** ptr);
/* Host FP64 copy of an auxiliary field: (Nx, Ny) dense, or [Nz][Ny][Nx] dense for centre fields. */
int obgc_pisces_model_read_field(obgc_pisces_model* m, int32_t which, double* out);
/* CUDA events around each stage's phases of the next obgc_pisces_model_step calls (on: nonzero). */
int obgc_pisces_model_set_profiling(obgc_pisces_model* m, int32_t on);
/* Device milliseconds of the last profiled step call, summed over its stages: ms[0] negatives +
 * light + euphotic depth + mixed-layer PAR, ms[1] calcite saturation, ms[2] the PISCES functor,
 * ms[3] the fused advection/RK3 substep.  *stages = RK3 stages timed. */
int obgc_pisces_model_last_timing(obgc_pisces_model* m, double* ms, int32_t* stages);

/* ---------------------------------------------------------------------------------------------
 * Batched single-column runs.  Each column is the reference's one-dimensional setup
 * (examples/column.jl:41-66: RectilinearGrid(size = (1, 1, Nz)) + LOBSTER or NPZD +
 * ScalarDiffusivity(kappa(z)) with kappa(z) = 1e-2 (1 + tanh((z - MLD) / 10)) / 2 + 1e-4 at :34),
 * time-stepped with Oceananigans' RK3 and a vertically implicit diffusion solve; sinking follows
 * setup_velocity_fields (src/Utils/sinking_velocity_fields.jl:10-35) and the light is TwoBand with
 * a constant surface PAR (src/Light/2band.jl:1-33).  An alkalinity pulse stands in for the OAE
 * release forcing (examples/oae_experiment.jl:56-73) as an instantaneous addition at one level.
 * Replaces running one NonhydrostaticModel per column; the engine keeps every column resident on
 * the device, packs whole columns into thread blocks and advances all of them per launch.
 * ------------------------------------------------------------------------------------------- */
typedef struct obgc_columns obgc_columns;

#define OBGC_COLUMN_MAX_LEVELS 512

typedef struct obgc_column_spec {
    int32_t Nz;              /* levels, 1..OBGC_COLUMN_MAX_LEVELS                              */
    int32_t nsteps;          /* RK3 steps to run                                               */
    double dz;               /* level thickness (m)                                            */
    double dt;               /* step (s)                                                       */
    double surface_PAR;      /* constant surface PAR (W/m2)                                    */
    double mu0;              /* phytoplankton_maximum_growth_rate for this column (<= 0: model's) */
    int32_t pulse_step;      /* step at whose start pulse_amount is added to Alk (-1: none)    */
    int32_t pulse_k;         /* level of the pulse (0 = bottom)                                */
    double pulse_amount;     /* alkalinity added (meq/m3)                                      */
    double temperature;      /* T (degC) and S of the column's surface water, read by the CO2  */
    double salinity;         /* gas exchange (obgc_columns_desc.gas_exchange)                  */
} obgc_column_spec;

typedef struct obgc_columns_desc {
    obgc_npd_params npd;         /* NPZD, or LOBSTER with the carbonate system                 */
    obgc_twoband_params light;
    int32_t precision;           /* OBGC_PREC_F32, OBGC_PREC_F64, or OBGC_PREC_MIXED (FP64 state
                                    and diffusion solve, FP32 light / sinking / BGC)           */
    int32_t pack_cells;          /* cells per thread-block pack (0: 1024)                      */
    int32_t threads;             /* threads per block (0: 256)                                 */
    int32_t max_columns;         /* column slots                                               */
    int64_t arena_cells;         /* device cells reserved for column state (the HBM budget)    */
    int32_t negatives;           /* enum obgc_negatives                                        */
    uint32_t zero_exclude;       /* ZeroNegativeTracers exclude mask (bit n = enum obgc_tracer n) */
    double invalid_fill_value;   /* ScaleNegativeTracers fill for a negative group total (NaN) */
    /* FieldBoundaryConditions(top = CarbonDioxideGasExchangeBoundaryCondition()) on DIC of every
     * LOBSTER column (examples/column.jl:54-64): 1 on, 0 off.  `gas` (gas = OBGC_GAS_CO2, constant
     * wind speed and air concentration: no wind or air fields) gives the condition's coefficients;
     * each RK3 stage takes the flux from the column's surface DIC and Alk and its spec's
     * temperature and salinity, and the surface cell loses flux / dz. */
    int32_t gas_exchange;
    int32_t reserved1;
    obgc_gas_exchange gas;
} obgc_columns_desc;

int obgc_columns_create(const obgc_columns_desc* desc, obgc_columns** out);
int obgc_columns_destroy(obgc_columns* eng);
/* Tracer rows of a column's state, in required_biogeochemical_tracers order; returns the count. */
int obgc_columns_tracers(const obgc_columns* eng, int32_t* names, int32_t cap);
/* Add a column: init is host [n_tracers][Nz] (FP64), kappa host [Nz+1] face diffusivities (m2/s,
 * bottom first; the two wall faces are ignored: no flux).  OBGC_ERR_BUSY when no slot or arena
 * space is free. */
int obgc_columns_add(obgc_columns* eng, const obgc_column_spec* spec, const double* init,
                     const double* kappa, int64_t* slot);
/* One launch: every live column advances min(max_steps, its remaining steps). */
int obgc_columns_advance(obgc_columns* eng, int32_t max_steps, void* stream);
/* Advance every live column by min(nsteps, its remaining steps) through ceil(nsteps /
 * steps_per_launch) launches; with use_graph != 0 the launches are captured once into a CUDA graph
 * (cached until columns are added or removed) and replayed. */
int obgc_columns_run(obgc_columns* eng, int32_t nsteps, int32_t steps_per_launch, int32_t use_graph,
                     void* stream);
/* Remaining steps of a slot (0: finished). */
int obgc_columns_remaining(const obgc_columns* eng, int64_t slot, int32_t* steps_left);
/* Copy a slot's state to host [n_tracers][Nz] FP64 (synchronises the engine's last stream). */
int obgc_columns_read(obgc_columns* eng, int64_t slot, double* state);
int obgc_columns_remove(obgc_columns* eng, int64_t slot);
/* Autotune the launch shape on the live columns: time `steps` steps of candidate (threads, pack
 * cells) pairs (the pack size at 256 threads, then the block size at the best pack size, then the
 * neighbouring pack sizes; each from the same state, which is restored afterwards) and keep the
 * fastest; writes the choice to *threads / *pack_cells. */
int obgc_columns_autotune(obgc_columns* eng, int32_t steps, int32_t* threads, int32_t* pack_cells,
                          void* stream);

/* ---------------------------------------------------------------------------------------------
 * Continuous-batching column service.  Requests (one column run each) are submitted from any host
 * thread; a worker thread admits them into the column engine while a slot and arena space (the
 * HBM budget) are free, advances every resident run by chunk_steps per launch with two launches
 * queued, copies finished runs back behind their last launch, and frees their space for the next
 * requests.  A run's result does not depend on the runs it shares launches with.  This serving
 * layer has no counterpart in the reference, which runs one model per process
 * (examples/column.jl, examples/oae_experiment.jl).
 * ------------------------------------------------------------------------------------------- */
typedef struct obgc_service obgc_service;

typedef struct obgc_service_desc {
    obgc_columns_desc columns;   /* engine: model, precision, slots, arena (HBM budget)       */
    int32_t chunk_steps;         /* steps per launch (0: 32)                                  */
    int32_t max_queue;           /* queued requests before submit returns OBGC_ERR_BUSY (0: no limit) */
} obgc_service_desc;

typedef struct obgc_service_stats {
    int64_t submitted, admitted, completed, launches;
    double p50_ms, p99_ms, mean_ms, max_ms;   /* submit -> result available, completed requests  */
    double span_s;                            /* first submit -> last completion                 */
} obgc_service_stats;

/* Creates the engine and starts the worker on the calling thread's current device. */
int obgc_service_create(const obgc_service_desc* desc, obgc_service** out);
/* Stops the worker after the chunk in flight and frees everything (unfinished runs are dropped). */
int obgc_service_destroy(obgc_service* svc);
/* Queue a run: init host [n_tracers][Nz] FP64 and kappa [Nz+1] are copied; returns at once. */
int obgc_service_submit(obgc_service* svc, const obgc_column_spec* spec, const double* init,
                        const double* kappa, int64_t* request);
/* Block until the run has finished (OBGC_ERR_TIMEOUT after timeout_s); copies its final state
 * [n_tracers][Nz] and its latency, and forgets the request. */
int obgc_service_wait(obgc_service* svc, int64_t request, double timeout_s, double* state, double* latency_ms);
/* Block until every submitted run has finished. */
int obgc_service_drain(obgc_service* svc, double timeout_s);
int obgc_service_get_stats(obgc_service* svc, obgc_service_stats* out);
int obgc_service_reset_stats(obgc_service* svc);
/* The engine the worker drives (read-only use: its tracer list). */
int obgc_service_engine(obgc_service* svc, obgc_columns** engine);

#ifdef __cplusplus
}
#endif
#endif /* OBGC_H */
