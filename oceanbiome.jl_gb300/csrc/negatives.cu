// negatives.cu — ScaleNegativeTracers / ZeroNegativeTracers over 3-D fields, and the conserved
// groups of the NPD models.
#include <cstring>
#include "negatives.cuh"

namespace obgc {

int conserved_group(const obgc_npd_params& p, int group, int* names, double* scale) {
    int n = 0;
    auto add = [&](int name, double f) { names[n] = name; scale[n++] = f; };
    if (group == 0) {
        add(OBGC_P, 1);
        add(OBGC_Z, 1);
        if (p.nutrients == OBGC_NUT_NUTRIENT) add(OBGC_N, 1);
        else { add(OBGC_NO3, 1); add(OBGC_NH4, 1); }
        if (p.detritus == OBGC_DET_VARIABLE_REDFIELD) { add(OBGC_SPON, 1); add(OBGC_BPON, 1); add(OBGC_DON, 1); }
        else if (p.detritus == OBGC_DET_TWO_PARTICLE) { add(OBGC_SPOM, 1); add(OBGC_BPOM, 1); add(OBGC_DOM, 1); }
        else if (p.detritus == OBGC_DET_SINGLE) add(OBGC_D, 1);
        return n;
    }
    if (group != 1 || !p.carbonate_system) return -1;
    const double R = p.redfield_ratio, rho = p.carbon_calcite_ratio;
    add(OBGC_P, (1 + rho) * R);
    add(OBGC_Z, R);
    add(OBGC_DIC, 1);
    if (p.detritus == OBGC_DET_VARIABLE_REDFIELD) { add(OBGC_SPOC, 1); add(OBGC_BPOC, 1); add(OBGC_DOC, 1); }
    else if (p.detritus == OBGC_DET_TWO_PARTICLE) { add(OBGC_SPOM, R); add(OBGC_BPOM, R); add(OBGC_DOM, R); }
    else if (p.detritus == OBGC_DET_SINGLE) add(OBGC_D, R);
    return n;
}

int negatives_spec(const obgc_npd_params& p, int mode, int nt, const int* names, uint32_t zero_exclude, double fill,
                   NegativesSpec* out) {
    std::memset(out, 0, sizeof(*out));
    out->mode = mode;
    out->nt = nt;
    out->fill = fill;
    if (mode == OBGC_NEGATIVES_NONE) return OBGC_OK;
    if (nt > 32) return fail(OBGC_ERR_UNSUPPORTED, "negative-tracer modifier: more than 32 tracers");
    if (mode == OBGC_NEGATIVES_ZERO) {
        int passive = 0;
        for (int q = 0; q < nt; q++) {
            const int bit = names[q] >= 0 ? names[q] : OBGC_NUM_NAMED + passive++;
            if (bit < 32 && ((zero_exclude >> bit) & 1u)) out->zero_skip |= 1u << q;
        }
        return OBGC_OK;
    }
    if (mode != OBGC_NEGATIVES_SCALE) return fail(OBGC_ERR_INVALID_ARGUMENT, "negative-tracer modifier: unknown mode");
    for (int g = 0; g < NEG_MAX_GROUPS; g++) {
        int gnames[16];
        double f[16];
        const int n = conserved_group(p, g, gnames, f);
        if (n < 0) break;
        int m = 0;
        for (int k = 0; k < n && m < NEG_MAX_MEMBERS; k++)
            for (int q = 0; q < nt; q++)
                if (names[q] == gnames[k]) { out->slot[g][m] = q; out->fac[g][m] = f[k]; m++; break; }
        out->gn[g] = m;
        out->ng = g + 1;
    }
    return OBGC_OK;
}

template <typename T>
struct NegFields {
    T* f[NEG_MAX_FIELDS];
};

template <typename T>
__global__ void negatives_kernel(const __grid_constant__ NegFields<T> F, const __grid_constant__ NegativesSpec s, int Nx,
                                 int Ny, int Nz, int64_t sj, int64_t sk) {
    const int64_t N = (int64_t)Nx * Ny * Nz;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(c % Nx);
        const int64_t r = c / Nx;
        const int j = (int)(r % Ny), k = (int)(r / Ny);
        const int64_t o = i + j * sj + k * sk;
        negatives_cell<T>(s, [&](int q) -> T& { return F.f[q][o]; });
    }
}

int launch_negatives(const NegativesSpec& s, size_t elem, void* const* fields, const obgc_grid& g, cudaStream_t st) {
    if (s.mode == OBGC_NEGATIVES_NONE) return OBGC_OK;
    const int64_t N = (int64_t)g.Nx * g.Ny * g.Nz;
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (N + 255) / 256;
    const unsigned blocks = (unsigned)(want < (int64_t)sms * 8 ? want : (int64_t)sms * 8);
    if (elem == 4) {
        NegFields<float> F;
        for (int q = 0; q < NEG_MAX_FIELDS; q++) F.f[q] = q < s.nt ? static_cast<float*>(fields[q]) : nullptr;
        negatives_kernel<float><<<blocks, 256, 0, st>>>(F, s, g.Nx, g.Ny, g.Nz, g.stride_j, g.stride_k);
    } else {
        NegFields<double> F;
        for (int q = 0; q < NEG_MAX_FIELDS; q++) F.f[q] = q < s.nt ? static_cast<double*>(fields[q]) : nullptr;
        negatives_kernel<double><<<blocks, 256, 0, st>>>(F, s, g.Nx, g.Ny, g.Nz, g.stride_j, g.stride_k);
    }
    OBGC_LAUNCHED("negatives_kernel");
    return OBGC_OK;
}

}  // namespace obgc

using namespace obgc;

extern "C" int obgc_npd_conserved_tracers(const obgc_npd_params* p, int32_t group, int32_t* names, double* scalefactors,
                                          int32_t cap) {
    if (!p || !names || !scalefactors) return -OBGC_ERR_INVALID_ARGUMENT;
    int nm[16];
    double f[16];
    const int n = conserved_group(*p, group, nm, f);
    if (n < 0) return -OBGC_ERR_INVALID_ARGUMENT;
    if (n > cap) return -OBGC_ERR_INVALID_ARGUMENT;
    for (int q = 0; q < n; q++) { names[q] = nm[q]; scalefactors[q] = f[q]; }
    return n;
}

static int check_fields(const char* where, const obgc_grid* grid, int32_t dtype, int32_t n, void* const* fields) {
    if (!valid_grid(grid) || !fields || n < 1 || n > NEG_MAX_FIELDS || (dtype != OBGC_F32 && dtype != OBGC_F64))
        return fail(OBGC_ERR_INVALID_ARGUMENT, std::string(where) + ": bad argument");
    for (int q = 0; q < n; q++)
        if (!fields[q]) return fail(OBGC_ERR_INVALID_ARGUMENT, std::string(where) + ": null field");
    return OBGC_OK;
}

extern "C" int obgc_scale_negatives(const obgc_grid* grid, int32_t dtype, int32_t n_fields, void* const* fields,
                                    const double* scalefactors, double invalid_fill_value, void* stream) {
    int rc = check_fields("obgc_scale_negatives", grid, dtype, n_fields, fields);
    if (rc != OBGC_OK) return rc;
    if (n_fields > NEG_MAX_MEMBERS)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_scale_negatives: at most 8 tracers in a group");
    NegativesSpec s;
    std::memset(&s, 0, sizeof(s));
    s.mode = OBGC_NEGATIVES_SCALE;
    s.ng = 1;
    s.nt = n_fields;
    s.gn[0] = n_fields;
    s.fill = invalid_fill_value;
    for (int q = 0; q < n_fields; q++) {
        s.slot[0][q] = q;
        s.fac[0][q] = scalefactors ? scalefactors[q] : 1.0;
    }
    return launch_negatives(s, dtype == OBGC_F32 ? 4 : 8, fields, *grid, static_cast<cudaStream_t>(stream));
}

extern "C" int obgc_zero_negatives(const obgc_grid* grid, int32_t dtype, int32_t n_fields, void* const* fields,
                                   void* stream) {
    int rc = check_fields("obgc_zero_negatives", grid, dtype, n_fields, fields);
    if (rc != OBGC_OK) return rc;
    NegativesSpec s;
    std::memset(&s, 0, sizeof(s));
    s.mode = OBGC_NEGATIVES_ZERO;
    s.nt = n_fields;
    return launch_negatives(s, dtype == OBGC_F32 ? 4 : 8, fields, *grid, static_cast<cudaStream_t>(stream));
}
