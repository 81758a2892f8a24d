// budget_static.cu — the compensated tracer-budget reduction without any device allocation.
//
// Its scratch (one compensated partial sum per block, and the final total) is a file-scope
// __device__ array, so callers that cannot allocate device memory can still take a budget.  In host
// code the array's name is only a host-side stand-in, not a device address: the address is looked
// up per device with cudaGetSymbolAddress on that device's first call and handed to the kernels.
#include <mutex>
#include <vector>
#include "obgc_common.cuh"

namespace obgc {

struct SumPair {
    double s, c;   // Neumaier sum and compensation
};

static __device__ __align__(256) SumPair g_budget_partials[OBGC_BUDGET_STATIC_SLOTS];
static __device__ __align__(256) double g_budget_total;

namespace {

struct StaticScratch {
    SumPair* partials = nullptr;
    double* total = nullptr;
};

std::mutex g_scratch_mutex;
std::vector<StaticScratch> g_scratch;   // indexed by device ordinal

// Device addresses of the static scratch on the current device (looked up once per device).
int static_scratch(StaticScratch* out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if ((int)g_scratch.size() <= dev) g_scratch.resize(dev + 1);
    StaticScratch& s = g_scratch[dev];
    if (!s.partials) {
        void* p = nullptr;
        void* t = nullptr;
        e = cudaGetSymbolAddress(&p, g_budget_partials);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(budget partials)");
        e = cudaGetSymbolAddress(&t, g_budget_total);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(budget total)");
        s.partials = static_cast<SumPair*>(p);
        s.total = static_cast<double*>(t);
    }
    *out = s;
    return OBGC_OK;
}

__device__ __forceinline__ void pair_add(SumPair& a, double x) {
    const double t = a.s + x;
    if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
    else a.c += (x - t) + a.s;
    a.s = t;
}
__device__ __forceinline__ void pair_merge(SumPair& a, const SumPair& b) {
    pair_add(a, b.s);
    a.c += b.c;
}

constexpr int THREADS = 256;

template <typename TS>
struct StaticBudgetArgs {
    const TS* f[OBGC_BUDGET_STATIC_MAX_FIELDS];
    double scale[OBGC_BUDGET_STATIC_MAX_FIELDS];
    int n;
};

template <typename TS>
__global__ void __launch_bounds__(THREADS) static_budget_partial(StaticBudgetArgs<TS> b, int Nx, int Ny, int Nz,
                                                                 int64_t sj, int64_t sk, SumPair* __restrict__ partial) {
    const int64_t NN = (int64_t)Nx * Ny, N = NN * Nz;
    SumPair acc = {0.0, 0.0};
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < N; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t idx = (c % Nx) + ((c / Nx) % Ny) * sj + (c / NN) * sk;
        for (int q = 0; q < b.n; q++) pair_add(acc, b.scale[q] * (double)b.f[q][idx]);
    }
    __shared__ SumPair red[THREADS];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) pair_merge(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];   // every used slot is rewritten each call
}

__global__ void __launch_bounds__(THREADS) static_budget_final(const SumPair* __restrict__ partial, int n, double* total) {
    SumPair acc = {0.0, 0.0};
    for (int q = threadIdx.x; q < n; q += blockDim.x) pair_merge(acc, partial[q]);
    __shared__ SumPair red[THREADS];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) pair_merge(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = red[0].s + red[0].c;
}

template <typename TS>
int run_static_budget(const obgc_grid* g, int n, const void* const* fields, const double* scale, double* total,
                      cudaStream_t st) {
    StaticScratch s;
    int rc = static_scratch(&s);
    if (rc != OBGC_OK) return rc;
    StaticBudgetArgs<TS> b = {};
    b.n = n;
    for (int q = 0; q < n; q++) {
        if (!fields[q]) return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_tracer_budget_static: null field");
        b.f[q] = static_cast<const TS*>(fields[q]);
        b.scale[q] = scale[q];
    }
    int dev = 0, nsm = 152;
    OBGC_CUDA(cudaGetDevice(&dev));
    OBGC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const int64_t N = (int64_t)g->Nx * g->Ny * g->Nz;
    int64_t want = (N + THREADS - 1) / THREADS;
    int blocks = (int)(want < 4 * nsm ? want : 4 * nsm);
    if (blocks > OBGC_BUDGET_STATIC_SLOTS) blocks = OBGC_BUDGET_STATIC_SLOTS;
    if (blocks < 1) blocks = 1;
    static_budget_partial<TS><<<blocks, THREADS, 0, st>>>(b, g->Nx, g->Ny, g->Nz, g->stride_j, g->stride_k, s.partials);
    OBGC_LAUNCHED("static_budget_partial");
    static_budget_final<<<1, THREADS, 0, st>>>(s.partials, blocks, s.total);
    OBGC_LAUNCHED("static_budget_final");
    OBGC_CUDA(cudaMemcpyAsync(total, s.total, sizeof(double), cudaMemcpyDeviceToHost, st));
    OBGC_CUDA(cudaStreamSynchronize(st));
    return OBGC_OK;
}

}  // namespace
}  // namespace obgc

using namespace obgc;

extern "C" int obgc_tracer_budget_static(const obgc_grid* grid, int32_t dtype, int32_t n_fields, const void* const* fields,
                                         const double* scale, double* total, void* stream) {
    if (!valid_grid(grid) || !fields || !scale || !total || n_fields < 1)
        return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_tracer_budget_static: bad argument");
    if (n_fields > OBGC_BUDGET_STATIC_MAX_FIELDS)
        return fail(OBGC_ERR_INVALID_ARGUMENT,
                    "obgc_tracer_budget_static: at most " + std::to_string(OBGC_BUDGET_STATIC_MAX_FIELDS) +
                        " fields fit the static scratch, got " + std::to_string(n_fields));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (dtype == OBGC_F32) return run_static_budget<float>(grid, n_fields, fields, scale, total, st);
    if (dtype == OBGC_F64) return run_static_budget<double>(grid, n_fields, fields, scale, total, st);
    return fail(OBGC_ERR_INVALID_ARGUMENT, "obgc_tracer_budget_static: bad dtype");
}
