// step_inst.cu — one (precision, variant) slice of the fused substep kernels.  The build compiles
// this file once per slice with -DOBGC_INST_PREC=<0 f32 | 1 f64 | 2 mixed> -DOBGC_INST_V=<variant>,
// so the slices compile in parallel; each object registers its kernels with the dispatcher.
#include "step_launch.cuh"

#ifndef OBGC_INST_PREC
#define OBGC_INST_PREC 0
#endif
#ifndef OBGC_INST_V
#define OBGC_INST_V 1
#endif

namespace obgc {
namespace {

#if OBGC_INST_PREC == 0
typedef float TS_;
typedef float TC_;
#elif OBGC_INST_PREC == 1
typedef double TS_;
typedef double TC_;
#else
typedef double TS_;
typedef float TC_;
#endif

constexpr int V_ = OBGC_INST_V;
// tracer counts with a kernel: the BGC tracers alone, and followed by the carried T/S.  The
// external-tendency variant serves the PISCES groups of 9 and 8 of its 26 slots (every precision)
// and the passive tracers of every model (CarbonateSystem replicates included) in launches of 4,
// 2 and 1 tracers.
[[maybe_unused]] constexpr int NT_A = V_ == V_EXTERNAL ? 9 : n_bgc(V_);
[[maybe_unused]] constexpr int NT_B = V_ == V_NPZD ? 6 : V_ == V_EXTERNAL ? 8 : n_bgc(V_) + 2;

template <int NT>
int launch_fn(const void* a, int blocks, cudaStream_t st) {
    return launch_one<V_, NT, TS_, TC_>(*static_cast<const SubstepArgs<TS_, TC_>*>(a), blocks, st);
}
template <int NT>
int occupancy_fn(int* bps) { return occupancy_one<V_, NT, TS_, TC_>(bps); }

struct Registrar {
    Registrar() {
#if OBGC_INST_V == 5
        register_fused({OBGC_INST_PREC, V_, 1, &launch_fn<1>, &occupancy_fn<1>});
        register_fused({OBGC_INST_PREC, V_, 2, &launch_fn<2>, &occupancy_fn<2>});
        register_fused({OBGC_INST_PREC, V_, 4, &launch_fn<4>, &occupancy_fn<4>});
#endif
        register_fused({OBGC_INST_PREC, V_, NT_A, &launch_fn<NT_A>, &occupancy_fn<NT_A>});
        if (NT_B != NT_A) register_fused({OBGC_INST_PREC, V_, NT_B, &launch_fn<NT_B>, &occupancy_fn<NT_B>});
    }
};
Registrar registrar;

}  // namespace
}  // namespace obgc
