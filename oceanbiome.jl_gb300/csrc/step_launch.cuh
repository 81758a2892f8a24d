// step_launch.cuh — instantiation helpers for the fused substep kernel.  Each (precision, variant)
// slice is its own translation unit (step_inst.cu compiled once per slice) so they compile in
// parallel.
#pragma once
#include "step_kernel.cuh"

namespace obgc {

template <int V, int NT, typename TS, typename TC, bool EXT>
int ensure_configured() {
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(substep_kernel<V, NT, TS, TC, EXT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)substep_smem_bytes<TC, NT>());
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(substep_kernel)");
        configured = true;
    }
    return OBGC_OK;
}

// The lean instantiation unless the launch uses an optional term (substep_needs_ext).
template <int V, int NT, typename TS, typename TC>
int launch_one(const SubstepArgs<TS, TC>& a, int blocks, cudaStream_t st) {
    if (substep_needs_ext(a)) {
        const int rc = ensure_configured<V, NT, TS, TC, true>();
        if (rc != OBGC_OK) return rc;
        substep_kernel<V, NT, TS, TC, true><<<blocks, dim3(STEP_BX, STEP_BY), substep_smem_bytes<TC, NT>(), st>>>(a);
    } else {
        const int rc = ensure_configured<V, NT, TS, TC, false>();
        if (rc != OBGC_OK) return rc;
        substep_kernel<V, NT, TS, TC, false><<<blocks, dim3(STEP_BX, STEP_BY), substep_smem_bytes<TC, NT>(), st>>>(a);
    }
    OBGC_LAUNCHED("substep_kernel");
    return OBGC_OK;
}

// Blocks per SM (both instantiations share the launch bounds and shared memory; the larger one's
// figure is the one the persistent grid is sized by).
template <int V, int NT, typename TS, typename TC>
int occupancy_one(int* blocks_per_sm) {
    int rc = ensure_configured<V, NT, TS, TC, true>();
    if (rc == OBGC_OK) rc = ensure_configured<V, NT, TS, TC, false>();
    if (rc != OBGC_OK) return rc;
    int lean = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&lean, substep_kernel<V, NT, TS, TC, false>,
                                                                  STEP_BX * STEP_BY, substep_smem_bytes<TC, NT>());
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, substep_kernel<V, NT, TS, TC, true>,
                                                      STEP_BX * STEP_BY, substep_smem_bytes<TC, NT>());
    if (*blocks_per_sm > lean) *blocks_per_sm = lean;
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    return OBGC_OK;
}

// Registry of compiled fused kernels, filled by the step_inst.cu objects at load time.
typedef int (*fused_launch_fn)(const void* args, int blocks, cudaStream_t st);
typedef int (*fused_occupancy_fn)(int* blocks_per_sm);
struct FusedEntry {
    int prec, V, NT;
    fused_launch_fn launch;
    fused_occupancy_fn occupancy;
};
void register_fused(const FusedEntry& e);
const FusedEntry* find_fused(int prec, int V, int NT);

}  // namespace obgc
