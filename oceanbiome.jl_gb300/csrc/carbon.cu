// carbon.cu — batched FP64 carbonate-system solve (one thread per cell) and its host twin.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>
#include "carbon_device.cuh"

namespace obgc {

template <typename T>
__device__ __forceinline__ double opt_ld(const T* p, int64_t i) { return p ? (double)p[i] : 0.0; }

template <typename T>
__global__ void __launch_bounds__(128) carbon_kernel(obgc_carbon_options o, int64_t n, const T* __restrict__ DIC,
                                                     const T* __restrict__ Alk, const T* __restrict__ Tc,
                                                     const T* __restrict__ S, const T* __restrict__ Si,
                                                     const T* __restrict__ PO4, const T* __restrict__ P,
                                                     const T* __restrict__ pH, double* __restrict__ H_inout,
                                                     double* __restrict__ out, int32_t* __restrict__ iters,
                                                     int* __restrict__ failures) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const double H0 = (o.warm_start && H_inout && H_inout[c] > 0) ? H_inout[c] : exp(-2.302585092994046 * o.initial_pH_guess);
    double H;
    int it;
    bool ok;
    out[c] = carbon_cell(o, (double)DIC[c], (double)Alk[c], (double)Tc[c], (double)S[c], opt_ld(Si, c), opt_ld(PO4, c),
                         opt_ld(P, c), opt_ld(pH, c), H0, &H, &it, &ok);
    if (H_inout) H_inout[c] = H;
    if (iters) iters[c] = it;
    if (!ok) atomicAdd(failures, 1);
}

// One device int per GPU for the non-convergence count (allocated once per device).
static int* failure_counter(int dev) {
    static std::mutex m;
    static std::vector<int*> per_dev;
    std::lock_guard<std::mutex> g(m);
    if ((int)per_dev.size() <= dev) per_dev.resize(dev + 1, nullptr);
    if (!per_dev[dev]) {
        int* p = nullptr;
        if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
        per_dev[dev] = p;
    }
    return per_dev[dev];
}

template <typename T>
static int launch_carbon(const obgc_carbon_options* o, int64_t n, const void* DIC, const void* Alk, const void* T_,
                         const void* S, const void* Si, const void* PO4, const void* P, const void* pH, double* H,
                         double* out, int32_t* iters, cudaStream_t st) {
    int dev = 0;
    OBGC_CUDA(cudaGetDevice(&dev));
    int* fails = failure_counter(dev);
    if (!fails) return fail(OBGC_ERR_OUT_OF_MEMORY, "obgc_carbon_chemistry: counter allocation failed");
    OBGC_CUDA(cudaMemsetAsync(fails, 0, sizeof(int), st));
    const int blocks = (int)((n + 127) / 128);
    carbon_kernel<T><<<blocks, 128, 0, st>>>(*o, n, (const T*)DIC, (const T*)Alk, (const T*)T_, (const T*)S,
                                             (const T*)Si, (const T*)PO4, (const T*)P, (const T*)pH, H, out, iters, fails);
    OBGC_LAUNCHED("carbon_kernel");
    int hf = 0;
    OBGC_CUDA(cudaMemcpyAsync(&hf, fails, sizeof(int), cudaMemcpyDeviceToHost, st));
    OBGC_CUDA(cudaStreamSynchronize(st));
    if (hf) return fail(OBGC_ERR_NOT_CONVERGED, std::to_string(hf) + " cells did not converge");
    return OBGC_OK;
}

static bool valid_options(const obgc_carbon_options* o) {
    return o && o->output >= 0 && o->output <= OBGC_OUT_OMEGA_CALCITE && o->density >= OBGC_DENSITY_EOS80 &&
           o->density <= OBGC_DENSITY_TEOS10_POLYNOMIAL && o->max_iters >= 0 &&
           (o->density != OBGC_DENSITY_CONSTANT || o->density_value > 0);
}

}  // namespace obgc

using namespace obgc;

extern "C" int obgc_carbon_default_options(obgc_carbon_options* o) {
    if (!o) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_carbon_default_options: null");
    std::memset(o, 0, sizeof(*o));
    o->output = OBGC_OUT_FCO2;
    o->density = OBGC_DENSITY_TEOS10_POLYNOMIAL;
    o->max_iters = 100;
    o->initial_pH_guess = 8.0;
    o->atol = 1e-20;
    o->damping = 0.5;
    o->armijo_constant = 0.5;
    o->min_damping = std::pow(0.5, 10);
    o->calcium_ion_per_salinity = 0.0103 / 35;
    return OBGC_OK;
}

extern "C" int obgc_carbon_chemistry(const obgc_carbon_options* opt, int64_t n, int32_t dtype, const void* DIC,
                                     const void* Alk, const void* T, const void* S, const void* silicate,
                                     const void* phosphate, const void* P, const void* pH, double* H_inout, double* out,
                                     int32_t* iters, void* stream) {
    if (!valid_options(opt) || n < 0 || !DIC || !T || !S || !out || (!opt->ph_given && !Alk) ||
        (opt->ph_given && !pH) || (opt->has_pressure && !P))
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_carbon_chemistry: bad argument");
    if (n == 0) return OBGC_OK;
    const void* A = Alk ? Alk : DIC;   // Alk unused when pH is given
    cudaStream_t st = (cudaStream_t)stream;
    if (dtype == OBGC_F32) return launch_carbon<float>(opt, n, DIC, A, T, S, silicate, phosphate, P, pH, H_inout, out, iters, st);
    if (dtype == OBGC_F64) return launch_carbon<double>(opt, n, DIC, A, T, S, silicate, phosphate, P, pH, H_inout, out, iters, st);
    return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_carbon_chemistry: bad dtype");
}

extern "C" int obgc_carbon_chemistry_point(const obgc_carbon_options* opt, double DIC, double Alk, double T, double S,
                                           double silicate, double phosphate, double P, double pH, double* out) {
    if (!valid_options(opt) || !out) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_carbon_chemistry_point: bad argument");
    bool ok = true;
    *out = carbon_cell(*opt, DIC, Alk, T, S, silicate, phosphate, P, pH, std::exp(-2.302585092994046 * opt->initial_pH_guess),
                       nullptr, nullptr, &ok);
    return ok ? OBGC_OK : fail(OBGC_ERR_NOT_CONVERGED, "obgc_carbon_chemistry_point: solve did not converge");
}
