// step_launch.cuh — instantiation helpers for the fused substep kernel.  Each (precision, variant)
// slice is its own translation unit (step_inst.cu compiled once per slice) so they compile in
// parallel.
#pragma once
#include "step_kernel.cuh"

namespace obgc {

template <int V, int NT, typename TS, typename TC, bool EXT, int MODE = 0>
int ensure_configured() {
    static bool configured = false;
    if (!configured) {
        cudaError_t e = cudaFuncSetAttribute(substep_kernel<V, NT, TS, TC, EXT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)substep_smem_bytes<TC, NT, MODE != 0>());
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(substep_kernel)");
        configured = true;
    }
    return OBGC_OK;
}

// The lean instantiation unless the launch uses an optional term (substep_needs_ext); for the
// TMA-staged steps (FP32, lean) MODE 2 (tensor copies).
template <int V, int NT, typename TS, typename TC>
int launch_one(const SubstepArgs<TS, TC>& a, int blocks, cudaStream_t st) {
    const dim3 block(STEP_BX, STEP_BY);
    if (substep_needs_ext(a)) {
        if (a.tma_layout) return fail(OBGC_ERR_UNSUPPORTED, "substep: TMA staging needs the lean kernel");
        const int rc = ensure_configured<V, NT, TS, TC, true>();
        if (rc != OBGC_OK) return rc;
        substep_kernel<V, NT, TS, TC, true><<<blocks, block, substep_smem_bytes<TC, NT>(), st>>>(a);
    } else {
        bool done = false;
        if (a.tma_layout && (a.drift_mask & ((1u << window_a(V)) | (1u << window_b(V)))) && !a.fz_pre)
            return fail(OBGC_ERR_UNSUPPORTED, "substep: TMA staging needs the sinking fluxes of sink_flux_kernel");
        if constexpr (sizeof(TC) == 4) {   // FP32 and mixed
            if (a.tma_layout) {
                const int rc = ensure_configured<V, NT, TS, TC, false, 2>();
                if (rc != OBGC_OK) return rc;
                substep_kernel<V, NT, TS, TC, false, 2><<<blocks, block, substep_smem_bytes<TC, NT, true>(), st>>>(a);
                done = true;
            }
        }
        if (!done) {
            if (a.tma_layout) return fail(OBGC_ERR_UNSUPPORTED, "substep: TMA staging needs FP32 arithmetic");
            const int rc = ensure_configured<V, NT, TS, TC, false>();
            if (rc != OBGC_OK) return rc;
            substep_kernel<V, NT, TS, TC, false><<<blocks, block, substep_smem_bytes<TC, NT>(), st>>>(a);
        }
    }
    OBGC_LAUNCHED("substep_kernel");
    return OBGC_OK;
}

// Blocks per SM (the instantiations share the launch bounds; the smallest figure among them is the
// one the persistent grid is sized by).
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
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if (*blocks_per_sm > lean) *blocks_per_sm = lean;
    if constexpr (sizeof(TC) == 4) {
        rc = ensure_configured<V, NT, TS, TC, false, 2>();
        if (rc != OBGC_OK) return rc;
        int m2 = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&m2, substep_kernel<V, NT, TS, TC, false, 2>,
                                                          STEP_BX * STEP_BY, substep_smem_bytes<TC, NT, true>());
        if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
        if (*blocks_per_sm > m2) *blocks_per_sm = m2;
    }
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
