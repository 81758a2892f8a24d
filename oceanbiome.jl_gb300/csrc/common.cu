// common.cu — error reporting, launch accounting and ABI introspection of libobgc.so.
#include <atomic>
#include <cstddef>
#include <cstring>
#include "obgc_common.cuh"

namespace obgc {

static thread_local std::string g_last_error;
static std::atomic<int64_t> g_launches{0};

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int status, const std::string& msg) {
    g_last_error = msg;
    return status;
}
int cuda_fail(cudaError_t e, const char* where) {
    g_last_error = std::string(where) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return e == cudaErrorMemoryAllocation ? OBGC_ERR_OUT_OF_MEMORY
         : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? OBGC_ERR_NO_DEVICE : OBGC_ERR_CUDA;
}
void count_launches(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

}  // namespace obgc

extern "C" int obgc_abi_version(void) { return OBGC_ABI_VERSION; }
extern "C" const char* obgc_last_error_message(void) { return obgc::g_last_error.c_str(); }
extern "C" int64_t obgc_kernel_launch_count(void) { return obgc::g_launches.load(); }

// Size and field offsets of the ABI structs, so a binding (ctypes, Julia) can verify its mirror.
// which: 0 npd_params, 1 twoband, 2 surface, 3 grid, 4 carbon_options, 5 model_desc, 6 fields.
// out[0] = sizeof, out[1..] = offsets of selected fields.
extern "C" int obgc_struct_layout(int32_t which, int64_t* out, int32_t cap) {
    if (!out || cap < 4) return OBGC_ERR_INVALID_ARGUMENT;
    switch (which) {
        case 0: out[0] = sizeof(obgc_npd_params); out[1] = offsetof(obgc_npd_params, nitrification_rate);
                out[2] = offsetof(obgc_npd_params, phytoplankton_sinking_speed);
                out[3] = offsetof(obgc_npd_params, nitrification_oxygen_nitrogen_ratio); return 0;
        case 1: out[0] = sizeof(obgc_twoband_params); out[1] = offsetof(obgc_twoband_params, chlorophyll_red_exponent);
                out[2] = offsetof(obgc_twoband_params, pigment_ratio);
                out[3] = offsetof(obgc_twoband_params, phytoplankton_chlorophyll_ratio); return 0;
        case 2: out[0] = sizeof(obgc_surface); out[1] = offsetof(obgc_surface, value);
                out[2] = offsetof(obgc_surface, field); out[3] = 0; return 0;
        case 3: out[0] = sizeof(obgc_grid); out[1] = offsetof(obgc_grid, Lx);
                out[2] = offsetof(obgc_grid, stride_j); out[3] = offsetof(obgc_grid, stride_k); return 0;
        case 4: out[0] = sizeof(obgc_carbon_options); out[1] = offsetof(obgc_carbon_options, density_value);
                out[2] = offsetof(obgc_carbon_options, atol);
                out[3] = offsetof(obgc_carbon_options, calcium_ion_per_salinity); return 0;
        case 5: out[0] = sizeof(obgc_model_desc); out[1] = offsetof(obgc_model_desc, surface);
                out[2] = offsetof(obgc_model_desc, grid); out[3] = offsetof(obgc_model_desc, invalid_fill_value); return 0;
        case 6: out[0] = sizeof(obgc_fields); out[1] = offsetof(obgc_fields, passive);
                out[2] = offsetof(obgc_fields, u); out[3] = offsetof(obgc_fields, G); return 0;
        case 7: out[0] = sizeof(obgc_column_spec); out[1] = offsetof(obgc_column_spec, dz);
                out[2] = offsetof(obgc_column_spec, pulse_step); out[3] = offsetof(obgc_column_spec, pulse_amount); return 0;
        case 9: out[0] = sizeof(obgc_pisces_params); out[1] = offsetof(obgc_pisces_params, micro);
                out[2] = offsetof(obgc_pisces_params, doc_aggregation); out[3] = offsetof(obgc_pisces_params, open_bottom); return 0;
        case 10: out[0] = sizeof(obgc_pisces_phyto); out[1] = offsetof(obgc_pisces_phyto, exudated_fraction);
                 out[2] = offsetof(obgc_pisces_phyto, base_growth_rate); out[3] = offsetof(obgc_pisces_phyto, silicate_half_saturation_parameter); return 0;
        case 11: out[0] = sizeof(obgc_pisces_field); out[1] = offsetof(obgc_pisces_field, value);
                 out[2] = offsetof(obgc_pisces_field, data); out[3] = 0; return 0;
        case 8: out[0] = sizeof(obgc_columns_desc); out[1] = offsetof(obgc_columns_desc, light);
                out[2] = offsetof(obgc_columns_desc, arena_cells); out[3] = offsetof(obgc_columns_desc, invalid_fill_value); return 0;
    }
    return OBGC_ERR_INVALID_ARGUMENT;
}
