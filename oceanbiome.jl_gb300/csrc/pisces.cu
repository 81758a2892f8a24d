// pisces.cu — PISCES on the GPU: all tendencies of a cell per thread, the mixed-layer means of
// update_biogeochemical_state! and the calcite saturation with the pressure of the cell's depth.
#include <cmath>
#include <cstring>
#include "carbon_device.cuh"
#include "pisces_device.cuh"

namespace obgc {

// CBMDayLength (src/Utils/Utils.jl:18-34): day length (s) at latitude phi, t seconds into the year.
double cbm_day_length(double coefficient, double t, double phi) {
    const double day = 86400.0, deg = 3.141592653589793 / 180.0;
    double m = std::fmod(t, 365.0 * day);
    if (m < 0) m += 365.0 * day;
    const double J = std::floor(m / day);
    const double theta = 0.216310 + 2 * std::atan(0.9671396 * std::tan(0.00860 * (J - 186)));
    const double decl = std::asin(0.39795 * std::cos(theta)) / deg;
    auto sind = [&](double x) { return std::sin(std::fmod(x, 360.0) * deg); };
    auto cosd = [&](double x) { return std::cos(std::fmod(x, 360.0) * deg); };
    double L = (sind(coefficient) + sind(phi) * sind(decl)) / (cosd(phi) * cosd(decl));
    L = L != L ? L : (L > 1 ? 1.0 : (L < -1 ? -1.0 : L));
    return (24 - 24.0 / 180 * (std::acos(L) / deg)) * 3600.0;
}

// The two day lengths of one evaluation at model time t (growth_rate.jl:29 and :144).
PiscesClock<double> pisces_clock(const obgc_pisces_params& p, double t) {
    PiscesClock<double> c;
    c.day_length_growth = cbm_day_length(p.day_length_coefficient, p.latitude, t);
    c.day_length_ratio = cbm_day_length(p.day_length_coefficient, t, p.latitude);
    return c;
}

struct AuxField {
    int kind;
    double value;
    const void* data;
};

// Tracers and auxiliary fields in the state precision TS, tendencies in the compute precision TC.
template <typename TS, typename TC>
struct PiscesFields {
    const TS* tr[OBGC_PIS_NUM];
    TC* G[OBGC_PIS_NUM_BGC];
    AuxField aux[OBGC_PAUX_NUM];
};

// xy: dense (Nx, Ny) index i + j Nx; o: the cell with the grid's strides; k: level.
template <typename TS, typename TC>
__device__ __forceinline__ TC aux_at(const AuxField& f, int64_t xy, int64_t o, int64_t sk, int k) {
    switch (f.kind) {
        case OBGC_PF_XY: return TC(static_cast<const TS*>(f.data)[xy]);
        case OBGC_PF_XYZ: return TC(static_cast<const TS*>(f.data)[o]);
        case OBGC_PF_ZFACE: {
            const TS* w = static_cast<const TS*>(f.data);
            return TC(TS(0.5) * (w[o] + w[o + sk]));
        }
        case OBGC_PF_ZPROFILE: {
            const TS* w = static_cast<const TS*>(f.data);
            return TC(TS(0.5) * (w[k] + w[k + 1]));
        }
        default: return TC(f.value);
    }
}

// Sinking velocities of the reference's setup (sinking_velocity_fields.jl:10-35 for POC,
// DepthDependantSinkingSpeed common.jl:46-56 for GOC) at the faces of cell k, interpolated to its
// centre (the ℑz of two_size_class.jl:95-98).
template <typename T>
__device__ __forceinline__ T poc_face(const PiscesT<T>& p, int f, int Nz) {
    if (f >= Nz) return T(0);
    return -p.w_poc * (p.open_bottom ? T(1) : T(1) - t_exp(T(-f) / T(2)));
}
template <typename T>
__device__ __forceinline__ T goc_face(const PiscesT<T>& p, int f, int Nz, T dz, T Lz, T zmxl, T zeu) {
    if (f >= Nz) return T(0);
    const T zc = -Lz + (T(f) + T(0.5)) * dz;   // the face takes the centre depth of cell f
    return -p.w_goc_min + (p.w_goc_max - p.w_goc_min) * jmin(T(0), zc - jmin(zmxl, zeu)) / T(5000);
}

template <typename TS, typename T>
__global__ void __launch_bounds__(128) pisces_kernel(const __grid_constant__ PiscesT<T> p,
                                                    const __grid_constant__ PiscesFields<TS, T> F, int Nx, int Ny, int Nz,
                                                    int64_t sj, int64_t sk, T dz, T Lz, const PiscesClock<T> clk) {
    const int64_t N = (int64_t)Nx * Ny * Nz;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % Nx);
        const int64_t r = c / Nx;
        const int j = (int)(r % Ny), k = (int)(r / Ny);
        const int64_t xy = i + (int64_t)j * Nx, o = i + j * sj + k * sk;
        T v[OBGC_PIS_NUM], a[OBGC_PAUX_NUM], G[OBGC_PIS_NUM_BGC];
#pragma unroll
        for (int q = 0; q < OBGC_PIS_NUM; q++) v[q] = T(F.tr[q][o]);
#pragma unroll
        for (int q = 0; q < OBGC_PAUX_NUM; q++) a[q] = aux_at<TS, T>(F.aux[q], xy, o, sk, k);
        if (F.aux[OBGC_PAUX_WPOC].kind == OBGC_PF_AUTO)
            a[OBGC_PAUX_WPOC] = T(0.5) * (poc_face(p, k, Nz) + poc_face(p, k + 1, Nz));
        if (F.aux[OBGC_PAUX_WGOC].kind == OBGC_PF_AUTO)
            a[OBGC_PAUX_WGOC] = T(0.5) * (goc_face(p, k, Nz, dz, Lz, a[OBGC_PAUX_ZMXL], a[OBGC_PAUX_ZEU]) +
                                          goc_face(p, k + 1, Nz, dz, Lz, a[OBGC_PAUX_ZMXL], a[OBGC_PAUX_ZEU]));
        const T z = -Lz + (T(k) + T(0.5)) * dz;
        pisces_tendencies<T>(p, v, a, z, clk, G);
#pragma unroll
        for (int q = 0; q < OBGC_PIS_NUM_BGC; q++) F.G[q][o] = G[q];
    }
}

// _compute_mixed_layer_mean! (mean_mixed_layer_properties.jl:25-46): one thread per column.
template <typename T>
__global__ void mixed_layer_mean_kernel(const T* __restrict__ C, AuxField zmxl, T* __restrict__ out, int Nx, int Ny, int Nz,
                                        int64_t sj, int64_t sk, T dz, T Lz) {
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= (int64_t)Nx * Ny) return;
    const int i = (int)(c % Nx), j = (int)(c / Nx);
    const int64_t oxy = i + j * sj;   // the column in the centre field
    const T zm = zmxl.kind == OBGC_PF_XY ? static_cast<const T*>(zmxl.data)[c] : T(zmxl.value);
    T sum = T(0), depth = T(0);
    for (int k = Nz - 1; k >= 0; k--) {
        const T zk = -Lz + T(k) * dz, zk1 = -Lz + T(k + 1) * dz;
        const T dzk = zk1 - zk;
        const T dzk1 = zk1 > zm ? zk1 - zm : T(0);
        const T d = zk >= zm ? dzk : dzk1;
        sum += C[oxy + k * sk] * d;
        depth += d;
    }
    out[c] = sum / depth;   // (Nx, Ny) output, dense
}

// _compute_calcite_saturation! (compute_calcite_saturation.jl:23-36): P from the depth of the cell.
template <typename T>
__global__ void __launch_bounds__(128) pisces_omega_kernel(obgc_carbon_options o, const T* DIC, const T* Alk, const T* Tc,
                                                          const T* S, const T* Si, T* out, int Nx, int Ny, int Nz, int64_t sj,
                                                          int64_t sk, double dz, double Lz, double* H_inout, int* failures) {
    const int64_t N = (int64_t)Nx * Ny * Nz;
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= N) return;
    const int i = (int)(c % Nx);
    const int64_t r = c / Nx;
    const int j = (int)(r % Ny), k = (int)(r / Ny);
    const int64_t off = i + j * sj + k * sk;
    const double z = -Lz + (k + 0.5) * dz;
    const double P = fabs(z) * 9.80665 * 1026 / 100000;
    double H;
    int it;
    bool ok;
    const double H0 = (H_inout && H_inout[c] > 0) ? H_inout[c] : exp(-2.302585092994046 * o.initial_pH_guess);
    out[off] = T(carbon_cell(o, (double)DIC[off], (double)Alk[off], (double)Tc[off], (double)S[off], Si ? (double)Si[off] : 0.0,
                             0.0, P, 0.0, H0, &H, &it, &ok));
    if (H_inout) H_inout[c] = H;
    if (!ok) atomicAdd(failures, 1);
}

}  // namespace obgc

using namespace obgc;

extern "C" int obgc_pisces_default_params(obgc_pisces_params* p) {
    if (!p) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_default_params: null");
    const double day = 86400.0;
    std::memset(p, 0, sizeof(*p));
    for (int c = 0; c < 2; c++) {
        obgc_pisces_phyto& ph = c ? p->diatoms : p->nano;
        const bool dia = c == 1;
        // MixedMondo / GrowthRespirationLimitedProduction / NitrogenIronPhosphateSilicateLimitation
        // defaults of MixedMondoNanoAndDiatoms (mixed_mondo_nano_diatoms.jl:1-30)
        ph.growth_kind = 1;
        ph.silicate_limited = dia;
        ph.exudated_fraction = 0.05;
        ph.blue_light_absorption = dia ? 1.6 : 2.1;
        ph.green_light_absorption = dia ? 0.69 : 0.42;
        ph.red_light_absorption = dia ? 0.7 : 0.4;
        ph.mortality_half_saturation = 0.2;
        ph.linear_mortality_rate = 0.01 / day;
        ph.base_quadratic_mortality = 0.01 / day;
        ph.maximum_quadratic_mortality = dia ? 0.03 / day : 0.0;
        ph.minimum_chlorophyll_ratio = 0.0033;
        ph.maximum_chlorophyll_ratio = dia ? 0.05 : 0.033;
        ph.maximum_iron_ratio = 0.06;
        ph.silicate_half_saturation = 2.0;
        ph.enhanced_silicate_half_saturation = 20.9;
        ph.optimal_silicate_ratio = 0.159;
        ph.half_saturation_for_iron_uptake = dia ? 3.0 : 1.0;
        ph.threshold_for_size_dependency = 1.0;
        ph.size_ratio = 3.0;
        ph.base_growth_rate = 0.6 / day;
        ph.temperature_sensitivity = 1.066;
        ph.dark_tolerance = (dia ? 4 : 3) * day;
        ph.initial_slope_of_PI_curve = 2.0;
        ph.low_light_adaptation = 0.0;
        ph.basal_respiration_rate = 0.033 / day;
        ph.reference_growth_rate = 1.0 / day;
        ph.minimum_ammonium_half_saturation = dia ? 0.039 : 0.013;
        ph.minimum_nitrate_half_saturation = dia ? 0.39 : 0.13;
        ph.minimum_phosphate_half_saturation = dia ? 2.4 : 0.8;
        ph.optimal_iron_quota = 0.007;
        ph.minimum_silicate_half_saturation = 1.0;
        ph.silicate_half_saturation_parameter = 16.6;
    }
    p->base_rain_ratio = 0.3;
    for (int c = 0; c < 2; c++) {
        obgc_pisces_zoo& z = c ? p->meso : p->micro;
        const bool meso = c == 1;
        // QualityDependantZooplankton defaults of MicroAndMesoZooplankton (zooplankton/defaults.jl:2-21)
        z.temperature_sensitivity = 1.079;
        z.maximum_grazing_rate = meso ? 0.75 / day : 3.0 / day;
        z.preference_P = meso ? 0.3 : 1.0;
        z.preference_D = meso ? 1.0 : 0.5;
        z.preference_POC = meso ? 0.3 : 0.1;
        z.preference_Z = meso ? 1.0 : 0.0;
        z.food_threshold_concentration = 0.3;
        z.specific_food_threshold_concentration = 0.001;
        z.grazing_half_saturation = 20.0;
        z.maximum_flux_feeding_rate = meso ? 2e3 / 1e6 : 0.0;
        z.iron_ratio = meso ? 0.015 : 0.01;
        z.minimum_growth_efficiency = meso ? 0.35 : 0.3;
        z.non_assimilated_fraction = 0.3;
        z.mortality_half_saturation = 0.2;
        z.quadratic_mortality = meso ? 0.03 / day : 0.004 / day;
        z.linear_mortality = meso ? 0.005 / day : 0.03 / day;
        z.dissolved_excretion_fraction = 0.6;
        z.undissolved_calcite_fraction = meso ? 0.75 : 0.5;
    }
    p->micro_bacteria = 0.7; p->meso_bacteria = 1.4; p->maximum_bacteria = 4.0; p->bacteria_depth_exponent = 0.684;
    p->doc_half_saturation_bacteria = 417.0; p->nitrate_half_saturation_bacteria = 0.03;
    p->ammonia_half_saturation_bacteria = 0.003; p->phosphate_half_saturation_bacteria = 0.003;
    p->iron_half_saturation_bacteria = 0.01;
    p->doc_remineralisation_rate = 0.3 / day; p->doc_bacteria_depth_exponent = 0.684; p->doc_reference_bacteria = 1.0;
    p->doc_temperature_sensitivity = 1.066;
    const double doc_a[5] = {0.37, 102, 3530, 5095, 114};
    for (int q = 0; q < 5; q++) p->doc_aggregation[q] = doc_a[q] * (1e-6 / day);
    p->pom_temperature_sensitivity = 1.066; p->pom_base_breakdown_rate = 0.025 / day;
    const double pom_a[4] = {25.9, 4452, 3.3, 47.1};
    for (int q = 0; q < 4; q++) p->pom_aggregation[q] = pom_a[q] * (1e-6 / day);
    p->minimum_iron_scavenging_rate = 3e-5 / day; p->load_specific_iron_scavenging_rate = 0.005 / day;
    p->bacterial_iron_uptake_efficiency = 0.16;
    p->small_fraction_bacterial_iron = 0.12 / 0.16; p->large_fraction_bacterial_iron = 0.04 / 0.16;
    p->base_liable_silicate_fraction = 0.5;
    p->fast_dissolution_rate_of_silicate = 0.025 / day; p->slow_dissolution_rate_of_silicate = 0.003 / day;
    p->base_calcite_dissolution_rate = 0.197 / day; p->calcite_dissolution_exponent = 1.0;
    p->maximum_iron_ratio_in_bacteria = 0.06; p->iron_half_saturation_for_bacteria = 0.3;
    p->maximum_bacterial_growth_rate = 0.6 / day;
    p->maximum_nitrification_rate = 0.05 / day; p->maximum_fixation_rate = 0.013 / day;
    p->iron_half_saturation_for_fixation = 0.1; p->phosphate_half_saturation_for_fixation = 0.8;
    p->light_saturation_for_fixation = 50.0;
    p->excess_scavenging_enhancement = 1000.0; p->maximum_ligand_concentration = 0.6; p->dissolved_ligand_ratio = 0.09;
    p->ratio_for_respiration = 133.0 / 122; p->ratio_for_nitrification = 32.0 / 122;
    p->first_anoxia_threshold = 6.0; p->second_anoxia_threshold = 1.0;
    p->nitrogen_redfield_ratio = 16.0 / 122; p->phosphate_redfield_ratio = 1.0 / 122;
    p->mixed_layer_shear = 1.0; p->background_shear = 0.01; p->latitude = 45.0; p->day_length_coefficient = 0.833;
    p->poc_sinking_speed = 2.0 / day;
    p->goc_minimum_speed = 30.0 / day; p->goc_maximum_speed = 200.0 / day; p->goc_maximum_depth = 5000.0;
    p->silicate_climatology = 7.5;
    p->open_bottom = 1;
    return OBGC_OK;
}

extern "C" int obgc_pisces_eval_point(const obgc_pisces_params* p, const double* values, const double* aux, double z, double t,
                                      double* G) {
    if (!p || !values || !aux || !G) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_eval_point: null argument");
    const PiscesT<double> P = make_pisces<double>(*p);
    pisces_tendencies<double>(P, values, aux, z, pisces_clock(*p, t), G);
    return OBGC_OK;
}

namespace {

bool valid_field(const obgc_pisces_field& f, int q) {
    if (f.kind == OBGC_PF_AUTO) return q == OBGC_PAUX_WPOC || q == OBGC_PAUX_WGOC;
    if (f.kind == OBGC_PF_CONSTANT) return true;
    return f.kind >= OBGC_PF_XY && f.kind <= OBGC_PF_ZPROFILE && f.kind != OBGC_PF_AUTO && f.data != nullptr;
}

}  // namespace

namespace obgc {

template <typename TS, typename T>
int launch_pisces(const obgc_pisces_params* p, const obgc_grid* g, const void* const* tracers, const obgc_pisces_field* aux,
                  void* const* G, double t, cudaStream_t st) {
    PiscesFields<TS, T> F;
    for (int q = 0; q < OBGC_PIS_NUM; q++) F.tr[q] = static_cast<const TS*>(tracers[q]);
    for (int q = 0; q < OBGC_PIS_NUM_BGC; q++) F.G[q] = static_cast<T*>(G[q]);
    for (int q = 0; q < OBGC_PAUX_NUM; q++) F.aux[q] = {aux[q].kind, aux[q].value, aux[q].data};
    const PiscesClock<double> c64 = pisces_clock(*p, t);
    const PiscesClock<T> clk{T(c64.day_length_growth), T(c64.day_length_ratio)};
    const int64_t N = (int64_t)g->Nx * g->Ny * g->Nz;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (N + 127) / 128;
    const unsigned blocks = (unsigned)(want < (int64_t)sms * 16 ? want : (int64_t)sms * 16);
    pisces_kernel<TS, T><<<blocks, 128, 0, st>>>(make_pisces<T>(*p), F, g->Nx, g->Ny, g->Nz, g->stride_j, g->stride_k,
                                                 T(g->Lz / g->Nz), T(g->Lz), clk);
    OBGC_LAUNCHED("pisces_kernel");
    return OBGC_OK;
}
template int launch_pisces<float, float>(const obgc_pisces_params*, const obgc_grid*, const void* const*,
                                         const obgc_pisces_field*, void* const*, double, cudaStream_t);
template int launch_pisces<double, float>(const obgc_pisces_params*, const obgc_grid*, const void* const*,
                                          const obgc_pisces_field*, void* const*, double, cudaStream_t);
template int launch_pisces<double, double>(const obgc_pisces_params*, const obgc_grid*, const void* const*,
                                           const obgc_pisces_field*, void* const*, double, cudaStream_t);

// Calcite saturation of every cell with the depth pressure, FP64 solve warm-started from H_inout.
template <typename T>
int launch_pisces_omega(const obgc_carbon_options* opt, const obgc_grid* grid, const void* DIC, const void* Alk,
                        const void* Tc, const void* S, const void* Si, void* Omega, double* H_inout, int* fails,
                        cudaStream_t st) {
    obgc_carbon_options o = *opt;
    o.output = OBGC_OUT_OMEGA_CALCITE;
    o.ph_given = 0;
    o.has_pressure = 1;
    const int64_t N = (int64_t)grid->Nx * grid->Ny * grid->Nz;
    pisces_omega_kernel<T><<<(unsigned)((N + 127) / 128), 128, 0, st>>>(
        o, (const T*)DIC, (const T*)Alk, (const T*)Tc, (const T*)S, (const T*)Si, (T*)Omega, grid->Nx, grid->Ny, grid->Nz,
        grid->stride_j, grid->stride_k, grid->Lz / grid->Nz, grid->Lz, H_inout, fails);
    OBGC_LAUNCHED("pisces_omega_kernel");
    return OBGC_OK;
}
template int launch_pisces_omega<float>(const obgc_carbon_options*, const obgc_grid*, const void*, const void*, const void*,
                                        const void*, const void*, void*, double*, int*, cudaStream_t);
template int launch_pisces_omega<double>(const obgc_carbon_options*, const obgc_grid*, const void*, const void*, const void*,
                                         const void*, const void*, void*, double*, int*, cudaStream_t);

}  // namespace obgc

extern "C" int obgc_pisces_tendencies(const obgc_pisces_params* p, const obgc_grid* grid, int32_t dtype,
                                      const void* const* tracers, const obgc_pisces_field* aux, void* const* G, double t,
                                      void* stream) {
    if (!p || !valid_grid(grid) || !tracers || !aux || !G || (dtype != OBGC_F32 && dtype != OBGC_F64))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_tendencies: bad argument");
    for (int q = 0; q < OBGC_PIS_NUM; q++)
        if (!tracers[q]) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_tendencies: a tracer field is NULL");
    for (int q = 0; q < OBGC_PIS_NUM_BGC; q++)
        if (!G[q]) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_tendencies: a tendency field is NULL");
    for (int q = 0; q < OBGC_PAUX_NUM; q++)
        if (!valid_field(aux[q], q)) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_tendencies: bad auxiliary field");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return dtype == OBGC_F32 ? launch_pisces<float, float>(p, grid, tracers, aux, G, t, st)
                             : launch_pisces<double, double>(p, grid, tracers, aux, G, t, st);
}

extern "C" int obgc_mixed_layer_mean(const obgc_grid* grid, int32_t dtype, const void* field, const obgc_pisces_field* zmxl,
                                     void* out, void* stream) {
    if (!valid_grid(grid) || !field || !zmxl || !out || (dtype != OBGC_F32 && dtype != OBGC_F64) ||
        (zmxl->kind != OBGC_PF_CONSTANT && !(zmxl->kind == OBGC_PF_XY && zmxl->data)))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_mixed_layer_mean: bad argument");
    const int64_t cols = (int64_t)grid->Nx * grid->Ny;
    const unsigned blocks = (unsigned)((cols + 127) / 128);
    const AuxField z{zmxl->kind, zmxl->value, zmxl->data};
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == OBGC_F32)
        mixed_layer_mean_kernel<float><<<blocks, 128, 0, st>>>(static_cast<const float*>(field), z, static_cast<float*>(out),
                                                               grid->Nx, grid->Ny, grid->Nz, grid->stride_j, grid->stride_k,
                                                               float(grid->Lz / grid->Nz), float(grid->Lz));
    else
        mixed_layer_mean_kernel<double><<<blocks, 128, 0, st>>>(static_cast<const double*>(field), z, static_cast<double*>(out),
                                                                grid->Nx, grid->Ny, grid->Nz, grid->stride_j, grid->stride_k,
                                                                grid->Lz / grid->Nz, grid->Lz);
    OBGC_LAUNCHED("mixed_layer_mean_kernel");
    return OBGC_OK;
}

extern "C" int obgc_pisces_calcite_saturation(const obgc_carbon_options* opt, const obgc_grid* grid, int32_t dtype,
                                              const void* DIC, const void* Alk, const void* T, const void* S, const void* Si,
                                              void* Omega, void* stream) {
    if (!opt || !valid_grid(grid) || !DIC || !Alk || !T || !S || !Omega || (dtype != OBGC_F32 && dtype != OBGC_F64))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_pisces_calcite_saturation: bad argument");
    obgc_carbon_options o = *opt;
    o.output = OBGC_OUT_OMEGA_CALCITE;
    o.ph_given = 0;
    o.has_pressure = 1;
    int* fails = nullptr;
    OBGC_CUDA(cudaMallocAsync((void**)&fails, sizeof(int), static_cast<cudaStream_t>(stream)));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    OBGC_CUDA(cudaMemsetAsync(fails, 0, sizeof(int), st));
    const int64_t N = (int64_t)grid->Nx * grid->Ny * grid->Nz;
    const unsigned blocks = (unsigned)((N + 127) / 128);
    if (dtype == OBGC_F32)
        pisces_omega_kernel<float><<<blocks, 128, 0, st>>>(o, (const float*)DIC, (const float*)Alk, (const float*)T, (const float*)S,
                                                           (const float*)Si, (float*)Omega, grid->Nx, grid->Ny, grid->Nz,
                                                           grid->stride_j, grid->stride_k, grid->Lz / grid->Nz, grid->Lz, nullptr, fails);
    else
        pisces_omega_kernel<double><<<blocks, 128, 0, st>>>(o, (const double*)DIC, (const double*)Alk, (const double*)T,
                                                            (const double*)S, (const double*)Si, (double*)Omega, grid->Nx,
                                                            grid->Ny, grid->Nz, grid->stride_j, grid->stride_k,
                                                            grid->Lz / grid->Nz, grid->Lz, nullptr, fails);
    OBGC_LAUNCHED("pisces_omega_kernel");
    int h = 0;
    OBGC_CUDA(cudaMemcpyAsync(&h, fails, sizeof(int), cudaMemcpyDeviceToHost, st));
    OBGC_CUDA(cudaFreeAsync(fails, st));
    OBGC_CUDA(cudaStreamSynchronize(st));
    if (h) return fail(OBGC_ERR_NOT_CONVERGED, std::to_string(h) + " cells did not converge");
    return OBGC_OK;
}
