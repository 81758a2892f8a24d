// negatives.cuh — the reference's negative-tracer modifiers, applied per cell.
//
// ScaleNegativeTracers (src/Utils/negative_tracers.jl:178-276): for each conserved group, the
// scaled total t = sum(c_q f_q) and the positive part p = sum(c_q f_q | c_q > 0) are accumulated in
// FP64 (the reference starts them from the Float64 literals 0.0); t < 0 becomes
// invalid_fill_value; then every member becomes c_q t / p when positive or non-finite, else 0.
// ZeroNegativeTracers (negative_tracers.jl:23-29): max(0, c) on every tracer not excluded (NaN
// stays NaN, as Julia's max propagates it).
#pragma once
#include "obgc_common.cuh"

namespace obgc {

constexpr int NEG_MAX_GROUPS = 5;
constexpr int NEG_MAX_MEMBERS = 10;
constexpr int NEG_MAX_FIELDS = 32;

struct NegativesSpec {
    int mode;                                    // OBGC_NEGATIVES_*
    int ng;                                      // conserved groups
    int nt;                                      // tracer slots (ZeroNegativeTracers)
    uint32_t zero_skip;                          // bit q: slot q is excluded from zeroing
    int gn[NEG_MAX_GROUPS];
    int slot[NEG_MAX_GROUPS][NEG_MAX_MEMBERS];
    double fac[NEG_MAX_GROUPS][NEG_MAX_MEMBERS];
    double fill;
};

// conserved_tracers (NutrientsPlanktonDetritus/coupling_utils.jl:1-52): names and scale factors
// of group 0 (nitrogen) or group 1 (carbon, only with the carbonate system; else returns -1).
int conserved_group(const obgc_npd_params& p, int group, int* names, double* scale);

// Build the spec for slots whose tracer names are `names[0..nt)` (-1: passive).  zero_exclude is a
// mask over tracer names (bit n: enum obgc_tracer n) and passive slots (bit 21 + passive index).
int negatives_spec(const obgc_npd_params& p, int mode, int nt, const int* names, uint32_t zero_exclude,
                   double fill, NegativesSpec* out);

// Apply the spec to one cell; ref(q) returns a reference to slot q's value.
template <typename T, typename Ref>
__device__ __forceinline__ void negatives_cell(const NegativesSpec& s, Ref&& ref) {
    if (s.mode == OBGC_NEGATIVES_SCALE) {
        for (int g = 0; g < s.ng; g++) {
            // separately rounded products and sums (no contraction), as the reference evaluates them
            double t = 0.0, p = 0.0;
            for (int m = 0; m < s.gn[g]; m++) {
                const T v = ref(s.slot[g][m]);
                const double x = __dmul_rn(double(v), s.fac[g][m]);
                t = __dadd_rn(t, x);
                if (v > T(0)) p = __dadd_rn(p, x);
            }
            t = t < 0.0 ? s.fill : t;
            for (int m = 0; m < s.gn[g]; m++) {
                T& v = ref(s.slot[g][m]);
                v = (!isfinite(v) || v > T(0)) ? T(__ddiv_rn(__dmul_rn(double(v), t), p)) : T(0);
            }
        }
    } else if (s.mode == OBGC_NEGATIVES_ZERO) {
        for (int q = 0; q < s.nt; q++) {
            if ((s.zero_skip >> q) & 1u) continue;
            T& v = ref(q);
            if (!(v > T(0)) && !isnan(v)) v = T(0);
        }
    }
}

// One pass over the interior of `nf` fields with the grid's strides (stream-ordered launch).
int launch_negatives(const NegativesSpec& s, size_t elem, void* const* fields, const obgc_grid& g, cudaStream_t st);

}  // namespace obgc
