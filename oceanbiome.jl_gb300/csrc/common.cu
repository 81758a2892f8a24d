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

namespace obgc {
// Eight independent FP64 FMA chains per thread: the FP64 pipe's issue rate, for the FP64 kernels'
// rooflines.  The result is stored only if it takes an impossible value, so the chains stay live.
__global__ void __launch_bounds__(256) fp64_fma_probe_kernel(double* out, int iters, double a, double b) {
    double x[8];
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = 1e-3 * (threadIdx.x + c);
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < 8; c++) x[c] = fma(x[c], a, b);
    }
    double sum = 0.0;
#pragma unroll
    for (int c = 0; c < 8; c++) sum += x[c];
    if (sum == -1.0) out[blockIdx.x] = sum;
}
}  // namespace obgc

extern "C" int obgc_fp64_fma_peak(double* gflops, void* stream) {
    if (!gflops) return obgc::fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_fp64_fma_peak: null output");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0, nsm = 0;
    OBGC_CUDA(cudaGetDevice(&dev));
    OBGC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = nsm * 8, threads = 256, iters = 4096;
    double* out = nullptr;
    OBGC_CUDA(cudaMallocAsync(&out, sizeof(double) * blocks, st));
    cudaEvent_t e0, e1;
    OBGC_CUDA(cudaEventCreate(&e0));
    OBGC_CUDA(cudaEventCreate(&e1));
    float best = 0.f;
    for (int r = 0; r < 4; r++) {
        cudaEventRecord(e0, st);
        obgc::fp64_fma_probe_kernel<<<blocks, threads, 0, st>>>(out, iters, 0.9999999, 1e-7);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (r > 0 && (best == 0.f || ms < best)) best = ms;   // the first run warms up
    }
    obgc::count_launches(4);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(out, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return obgc::cuda_fail(e, "obgc_fp64_fma_peak");
    *gflops = 2.0 * 8.0 * iters * (double)blocks * threads / (best * 1e-3) / 1e9;
    return OBGC_OK;
}

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
                out[3] = offsetof(obgc_carbon_options, saturation_mineral); return 0;
        case 5: out[0] = sizeof(obgc_model_desc); out[1] = offsetof(obgc_model_desc, surface);
                out[2] = offsetof(obgc_model_desc, grid); out[3] = offsetof(obgc_model_desc, passive_tendency_of); return 0;
        case 6: out[0] = sizeof(obgc_fields); out[1] = offsetof(obgc_fields, passive);
                out[2] = offsetof(obgc_fields, u); out[3] = offsetof(obgc_fields, G); return 0;
        case 7: out[0] = sizeof(obgc_column_spec); out[1] = offsetof(obgc_column_spec, dz);
                out[2] = offsetof(obgc_column_spec, pulse_step); out[3] = offsetof(obgc_column_spec, salinity); return 0;
        case 9: out[0] = sizeof(obgc_pisces_params); out[1] = offsetof(obgc_pisces_params, micro);
                out[2] = offsetof(obgc_pisces_params, doc_aggregation); out[3] = offsetof(obgc_pisces_params, open_bottom); return 0;
        case 10: out[0] = sizeof(obgc_pisces_phyto); out[1] = offsetof(obgc_pisces_phyto, exudated_fraction);
                 out[2] = offsetof(obgc_pisces_phyto, base_growth_rate); out[3] = offsetof(obgc_pisces_phyto, silicate_half_saturation_parameter); return 0;
        case 11: out[0] = sizeof(obgc_pisces_field); out[1] = offsetof(obgc_pisces_field, value);
                 out[2] = offsetof(obgc_pisces_field, data); out[3] = 0; return 0;
        case 12: out[0] = sizeof(obgc_gas_exchange); out[1] = offsetof(obgc_gas_exchange, wind_field);
                 out[2] = offsetof(obgc_gas_exchange, o2_solubility); out[3] = offsetof(obgc_gas_exchange, carbon); return 0;
        case 13: out[0] = sizeof(obgc_box_drivers); out[1] = offsetof(obgc_box_drivers, n_prescribed);
                 out[2] = offsetof(obgc_box_drivers, prescribed); out[3] = offsetof(obgc_box_drivers, forcing); return 0;
        case 8: out[0] = sizeof(obgc_columns_desc); out[1] = offsetof(obgc_columns_desc, light);
                out[2] = offsetof(obgc_columns_desc, arena_cells); out[3] = offsetof(obgc_columns_desc, gas); return 0;
    }
    return OBGC_ERR_INVALID_ARGUMENT;
}
