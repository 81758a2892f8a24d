// halo.cu — halo rows of a y slab: the pack and unpack kernels of the halo exchange between the
// ranks of a domain split in y (the ranks exchange the packed buffers with NCCL send/recv).
#include "obgc_common.cuh"

namespace obgc {
namespace {

constexpr int HALO_MAX_FIELDS = 32;

template <typename T>
struct HaloFields {
    T* f[HALO_MAX_FIELDS];
};

// One thread per buffer element of both directions: e = ((field Nz + k) halo + h) Nx + i, the south
// part first.  pack: buffer <- rows [halo + h] (south) and [Ny - 2 halo + h] (north); unpack: rows
// [h] <- south and [Ny - halo + h] <- north.
template <typename T, bool PACK>
__global__ void __launch_bounds__(256) halo_kernel(HaloFields<T> F, int n, int Nx, int Ny, int Nz, int64_t sj, int64_t sk,
                                                   int halo, T* __restrict__ south, T* __restrict__ north) {
    const int64_t per = (int64_t)n * Nz * halo * Nx;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < 2 * per; e += (int64_t)gridDim.x * blockDim.x) {
        const bool is_north = e >= per;
        const int64_t r = is_north ? e - per : e;
        const int i = (int)(r % Nx);
        const int h = (int)((r / Nx) % halo);
        const int k = (int)((r / ((int64_t)Nx * halo)) % Nz);
        const int q = (int)(r / ((int64_t)Nx * halo * Nz));
        T* buf = is_north ? north : south;
        int row;
        if (PACK) row = is_north ? Ny - 2 * halo + h : halo + h;
        else row = is_north ? Ny - halo + h : h;
        const int64_t idx = i + (int64_t)row * sj + (int64_t)k * sk;
        if (PACK) buf[r] = F.f[q][idx];
        else F.f[q][idx] = buf[r];
    }
}

template <typename T, bool PACK>
int launch_halo(const obgc_grid* g, int n, void* const* fields, int halo, void* south, void* north, cudaStream_t st) {
    HaloFields<T> F = {};
    for (int q = 0; q < n; q++) F.f[q] = static_cast<T*>(fields[q]);
    const int64_t total = 2 * (int64_t)n * g->Nz * halo * g->Nx;
    const int64_t want = (total + 255) / 256;
    const unsigned blocks = (unsigned)(want < 4096 ? want : 4096);
    halo_kernel<T, PACK><<<blocks, 256, 0, st>>>(F, n, g->Nx, g->Ny, g->Nz, g->stride_j, g->stride_k, halo,
                                                 static_cast<T*>(south), static_cast<T*>(north));
    OBGC_LAUNCHED(PACK ? "halo_pack_kernel" : "halo_unpack_kernel");
    return OBGC_OK;
}

int check_halo(const char* who, const obgc_grid* g, int32_t dtype, int32_t n, const void* const* fields, int32_t halo,
               const void* south, const void* north) {
    if (!valid_grid(g) || !fields || !south || !north || n < 1 || n > HALO_MAX_FIELDS || (dtype != OBGC_F32 && dtype != OBGC_F64))
        return fail(OBGC_ERR_INVALID_ARGUMENT, std::string(who) + ": bad argument");
    if (halo < 1 || g->Ny < 3 * halo)
        return fail(OBGC_ERR_INVALID_ARGUMENT, std::string(who) + ": a slab needs at least `halo` own rows between its halos");
    for (int q = 0; q < n; q++)
        if (!fields[q]) return fail(OBGC_ERR_INVALID_ARGUMENT, std::string(who) + ": null field");
    return OBGC_OK;
}

}  // namespace
}  // namespace obgc

using namespace obgc;

extern "C" int obgc_halo_pack(const obgc_grid* g, int32_t dtype, int32_t n, const void* const* fields, int32_t halo,
                              void* south, void* north, void* stream) {
    const int rc = check_halo("obgc_halo_pack", g, dtype, n, fields, halo, south, north);
    if (rc != OBGC_OK) return rc;
    void* const* f = const_cast<void* const*>(fields);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    return dtype == OBGC_F32 ? launch_halo<float, true>(g, n, f, halo, south, north, st)
                             : launch_halo<double, true>(g, n, f, halo, south, north, st);
}

extern "C" int obgc_halo_unpack(const obgc_grid* g, int32_t dtype, int32_t n, void* const* fields, int32_t halo,
                                const void* south, const void* north, void* stream) {
    const int rc = check_halo("obgc_halo_unpack", g, dtype, n, fields, halo, south, north);
    if (rc != OBGC_OK) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    void* s = const_cast<void*>(south);
    void* nn = const_cast<void*>(north);
    return dtype == OBGC_F32 ? launch_halo<float, false>(g, n, fields, halo, s, nn, st)
                             : launch_halo<double, false>(g, n, fields, halo, s, nn, st);
}
