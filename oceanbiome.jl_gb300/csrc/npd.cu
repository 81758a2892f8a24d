// npd.cu — NutrientsPlanktonDetritus model description (host) and the discrete-form tendency
// kernel of mode (i): every BGC tendency of every cell in one pass (replaces the per-tracer
// functor evaluation that Oceananigans inlines into one tendency kernel per tracer).
#include <cmath>
#include <cstring>
#include "npd_device.cuh"

namespace obgc {

static const double DAY = 86400.0;

// constructors.jl:65-96 (LOBSTER) and :177-227 (NPZD); @kwdef defaults of nutrients.jl:16-18,
// plankton.jl:19-58, detritus.jl:25-37,264-270, oxygen.jl:14-17.
static void lobster_defaults(obgc_npd_params* o) {
    std::memset(o, 0, sizeof(*o));
    o->nutrients = OBGC_NUT_NITRATE_AMMONIA;
    o->detritus = OBGC_DET_TWO_PARTICLE;
    o->light_limitation = OBGC_LIGHT_MONDO;
    o->phytoplankton_mortality_formulation = OBGC_QUADRATIC;
    o->grazing_concentration_formulation = OBGC_QUADRATIC;
    o->open_bottom = 1;
    o->nitrification_rate = 5.8e-7;
    o->nitrate_half_saturation = 0.7;
    o->ammonia_half_saturation = 0.001;
    o->iron_half_saturation = 2e-4;
    o->nitrate_ammonia_inhibition = 3.0;
    o->light_half_saturation = 33.0;
    o->phytoplankton_maximum_growth_rate = 2.42e-5;
    o->iron_ratio = 4.6375e-5;
    o->phytoplankton_exudation_fraction = 0.05;
    o->ammonia_fraction_of_exudate = 0.75;
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
    o->remineralisation_inorganic_fraction = 0.0;
    o->small_remineralisation_rate = 5.88e-7;
    o->large_remineralisation_rate = 5.88e-7;
    o->dissolved_remineralisation_rate = 3.86e-7;
    o->small_solid_waste_fraction = 0.5;
    o->detritus_redfield_ratio = 6.56;
    o->small_particle_sinking_speed = 3.47e-5;
    o->large_particle_sinking_speed = 200 / DAY;
    o->detritus_remineralisation_rate = 0.1213 / DAY;
    o->small_particle_fraction = 0.5;
    o->detritus_sinking_speed = 2.7489 / DAY;
    o->respiration_oxygen_nitrogen_ratio = 10.75;
    o->nitrification_oxygen_nitrogen_ratio = 2.0;
}

static void npzd_overrides(obgc_npd_params* o) {
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
}

static bool valid_params(const obgc_npd_params* p) {
    return p && p->nutrients >= 0 && p->nutrients <= 2 && p->detritus >= 0 && p->detritus <= 3 &&
           (p->carbonate_system == 0 || p->carbonate_system == 1) && (p->oxygen == 0 || p->oxygen == 1) &&
           (p->light_limitation == 0 || p->light_limitation == 1) &&
           (p->phytoplankton_mortality_formulation == 0 || p->phytoplankton_mortality_formulation == 1) &&
           (p->grazing_concentration_formulation == 0 || p->grazing_concentration_formulation == 1);
}

int required_tracers(const obgc_npd_params* p, int32_t* names) {
    int n = 0;
    if (p->nutrients == OBGC_NUT_NUTRIENT) names[n++] = OBGC_N;
    else {
        names[n++] = OBGC_NO3;
        names[n++] = OBGC_NH4;
        if (p->nutrients == OBGC_NUT_NITRATE_AMMONIA_IRON) names[n++] = OBGC_FE;
    }
    names[n++] = OBGC_P;
    names[n++] = OBGC_Z;
    if (p->has_temperature_coefficient) names[n++] = OBGC_T;
    if (p->detritus == OBGC_DET_TWO_PARTICLE) { names[n++] = OBGC_SPOM; names[n++] = OBGC_BPOM; names[n++] = OBGC_DOM; }
    else if (p->detritus == OBGC_DET_VARIABLE_REDFIELD) {
        names[n++] = OBGC_SPOC; names[n++] = OBGC_BPOC; names[n++] = OBGC_DOC;
        names[n++] = OBGC_SPON; names[n++] = OBGC_BPON; names[n++] = OBGC_DON;
    } else if (p->detritus == OBGC_DET_SINGLE) names[n++] = OBGC_D;
    if (p->carbonate_system) { names[n++] = OBGC_DIC; names[n++] = OBGC_ALK; }
    if (p->oxygen) names[n++] = OBGC_O2;
    return n;
}

// Scalar sinking speed of tracer `name` (0 if it has no drift velocity).
bool drift_speed(const obgc_npd_params* p, int name, double* w0) {
    const bool two = p->detritus == OBGC_DET_TWO_PARTICLE || p->detritus == OBGC_DET_VARIABLE_REDFIELD;
    const bool tp = p->detritus == OBGC_DET_TWO_PARTICLE;
    if (name == OBGC_P) { *w0 = p->phytoplankton_sinking_speed; return true; }
    if (name == OBGC_Z) { *w0 = p->zooplankton_sinking_speed; return true; }
    if (two && ((tp && name == OBGC_SPOM) || (!tp && (name == OBGC_SPON || name == OBGC_SPOC)))) {
        *w0 = p->small_particle_sinking_speed; return true;
    }
    if (two && ((tp && name == OBGC_BPOM) || (!tp && (name == OBGC_BPON || name == OBGC_BPOC)))) {
        *w0 = p->large_particle_sinking_speed; return true;
    }
    if (p->detritus == OBGC_DET_SINGLE && name == OBGC_D) { *w0 = p->detritus_sinking_speed; return true; }
    return false;
}

// setup_velocity_fields (src/Utils/sinking_velocity_fields.jl:10-35): faces 0..Nz-1 hold
// -w0 (open bottom) or -w0 (1 - exp(-f/2)); the surface face Nz is left at zero.
void drift_profile(double w0, int open_bottom, int Nz, double* w) {
    for (int f = 0; f < Nz; f++) w[f] = -w0 * (open_bottom ? 1.0 : (1 - std::exp(-(double)f / 2)));
    w[Nz] = 0.0;
}

template <typename T>
struct FieldTables {
    const T* f[OBGC_NUM_NAMED];
    T* g[OBGC_NUM_NAMED];
};

template <typename T>
__global__ void __launch_bounds__(256) tendencies_kernel(NPDParamsT<T> p, int Nx, int Ny, int Nz, int64_t sj,
                                                         int64_t sk, FieldTables<T> tb, const T* __restrict__ PAR,
                                                         uint32_t present, uint32_t wanted) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t NN = (int64_t)Nx * Ny;
    if (c >= NN * Nz) return;
    const int i = (int)(c % Nx);
    const int j = (int)((c / Nx) % Ny);
    const int k = (int)(c / NN);
    const int64_t idx = i + j * sj + k * sk;
    T v[OBGC_NUM_NAMED], g[OBGC_NUM_NAMED];
#pragma unroll
    for (int n = 0; n < OBGC_NUM_NAMED; n++) {
        v[n] = (present >> n) & 1u ? tb.f[n][idx] : T(0);
        g[n] = T(0);
    }
    npd_tendencies<V_RUNTIME, T>(p, v, PAR[idx], g);
#pragma unroll
    for (int n = 0; n < OBGC_NUM_NAMED; n++)
        if ((wanted >> n) & 1u) tb.g[n][idx] = g[n];
}

template <typename T>
static int launch_tendencies(const obgc_npd_params* p, const obgc_grid* g, const void* const* fields,
                             const void* PAR, void* const* G, cudaStream_t st) {
    int32_t names[32];
    const int n = required_tracers(p, names);
    uint32_t present = 0, wanted = 0;
    for (int q = 0; q < n; q++) {
        if (!fields[names[q]]) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_npd_tendencies: a required tracer field is NULL");
        if (G[names[q]]) wanted |= 1u << names[q];
    }
    for (int q = 0; q < OBGC_NUM_NAMED; q++)
        if (fields[q]) present |= 1u << q;
    FieldTables<T> tb;
    for (int q = 0; q < OBGC_NUM_NAMED; q++) { tb.f[q] = (const T*)fields[q]; tb.g[q] = (T*)G[q]; }
    const int64_t N = (int64_t)g->Nx * g->Ny * g->Nz;
    const int blocks = (int)((N + 255) / 256);
    tendencies_kernel<T><<<blocks, 256, 0, st>>>(make_params<T>(*p), g->Nx, g->Ny, g->Nz, g->stride_j, g->stride_k,
                                                 tb, (const T*)PAR, present, wanted);
    OBGC_LAUNCHED("tendencies_kernel");
    return OBGC_OK;
}

}  // namespace obgc

using namespace obgc;

extern "C" int obgc_npd_preset(int32_t preset, obgc_npd_params* out) {
    if (!out) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_npd_preset: null output");
    if (preset != OBGC_PRESET_LOBSTER && preset != OBGC_PRESET_NPZD)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_npd_preset: unknown preset");
    lobster_defaults(out);
    if (preset == OBGC_PRESET_NPZD) npzd_overrides(out);
    return OBGC_OK;
}

extern "C" int obgc_npd_required_tracers(const obgc_npd_params* p, int32_t* names, int32_t cap) {
    if (!valid_params(p) || !names) return -OBGC_ERR_INVALID_ARGUMENT;
    int32_t tmp[32];
    const int n = required_tracers(p, tmp);
    if (n > cap) return -OBGC_ERR_INVALID_ARGUMENT;
    std::memcpy(names, tmp, sizeof(int32_t) * n);
    return n;
}

extern "C" int obgc_npd_drift_velocity(const obgc_npd_params* p, int32_t name, int32_t Nz, double* w) {
    if (!valid_params(p) || Nz < 1 || !w || name < 0 || name >= OBGC_NUM_NAMED) return -OBGC_ERR_INVALID_ARGUMENT;
    double w0;
    if (!drift_speed(p, name, &w0)) return 0;
    drift_profile(w0, p->open_bottom, Nz, w);
    return 1;
}

extern "C" int obgc_npd_eval_point(const obgc_npd_params* p, int32_t name, double x, double y, double z,
                                   double t, const double* values, double PAR, double* out) {
    (void)x; (void)y; (void)z; (void)t;
    if (!valid_params(p) || !values || !out || name < 0 || name >= OBGC_NUM_NAMED)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_npd_eval_point: bad argument");
    double G[OBGC_NUM_NAMED] = {0};
    npd_tendencies<V_RUNTIME, double>(make_params<double>(*p), values, PAR, G);
    *out = G[name];
    return OBGC_OK;
}

extern "C" int obgc_npd_tendencies(const obgc_npd_params* p, const obgc_grid* grid, int32_t dtype,
                                   const void* const* fields, const void* PAR, void* const* G,
                                   double t, void* stream) {
    (void)t;
    if (!valid_params(p) || !valid_grid(grid) || !fields || !PAR || !G)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_npd_tendencies: bad argument");
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == OBGC_F32) return launch_tendencies<float>(p, grid, fields, PAR, G, st);
    if (dtype == OBGC_F64) return launch_tendencies<double>(p, grid, fields, PAR, G, st);
    return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_npd_tendencies: bad dtype");
}
