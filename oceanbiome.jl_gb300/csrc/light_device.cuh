// light_device.cuh — TwoBand PAR as a running column integral, shared by the standalone light
// kernel and the fused substep kernel (which marches its columns top-down and carries the sums).
//
// TwoBand (src/Light/2band.jl:15-32) on a uniform grid: the chlorophyll integral down to the
// centre of cell k is  dz * sum_{m>k} f(m) + dz/2 * f(k),  f(m) = (P_m Rchl / r)^e, and
//   PAR_k = PAR0 * (exp(k_r z_k - chi_r I_r) + exp(k_b z_k - chi_b I_b)) / 2.
#pragma once
#include "obgc_common.cuh"

namespace obgc {

template <typename T>
struct TwoBandT {
    T kr, kb, xr, xb, er, eb, inv_r_times_Rc;
};

template <typename T>
inline TwoBandT<T> make_twoband(const obgc_twoband_params& p) {
    TwoBandT<T> o;
    o.kr = T(p.water_red_attenuation); o.kb = T(p.water_blue_attenuation);
    o.xr = T(p.chlorophyll_red_attenuation); o.xb = T(p.chlorophyll_blue_attenuation);
    o.er = T(p.chlorophyll_red_exponent); o.eb = T(p.chlorophyll_blue_exponent);
    o.inv_r_times_Rc = T(p.phytoplankton_chlorophyll_ratio / p.pigment_ratio);
    return o;
}

// Chlorophyll terms of one cell: (P Rchl/r)^e_r and ^e_b, sharing one logarithm:
// c^e = 2^(e log2 c).  c = 0 gives 0 and c < 0 gives NaN, as the power does.
template <typename T>
__host__ __device__ __forceinline__ void twoband_terms(const TwoBandT<T>& L, T P, T& fr, T& fb) {
    const T c = P * L.inv_r_times_Rc;
#ifdef __CUDA_ARCH__
    const T l2 = sizeof(T) == 4 ? T(log2f(float(c))) : T(log2(double(c)));
    fr = sizeof(T) == 4 ? T(exp2f(float(L.er * l2))) : T(exp2(double(L.er * l2)));
    fb = sizeof(T) == 4 ? T(exp2f(float(L.eb * l2))) : T(exp2(double(L.eb * l2)));
#else
    fr = t_pow(c, L.er);
    fb = t_pow(c, L.eb);
#endif
}

// PAR at a cell centre z given the sums over the cells above (Sr, Sb) and this cell's terms.
template <typename T>
__host__ __device__ __forceinline__ T twoband_par(const TwoBandT<T>& L, T PAR0, T z, T dz, T Sr, T Sb,
                                                  T fr, T fb) {
    const T Ir = dz * Sr + T(0.5) * dz * fr;
    const T Ib = dz * Sb + T(0.5) * dz * fb;
    return PAR0 * (t_exp(L.kr * z - L.xr * Ir) + t_exp(L.kb * z - L.xb * Ib)) * T(0.5);
}

// default_surface_PAR (src/Light/Light.jl:45-47)
__host__ __device__ inline double default_surface_par(double t) {
    double c = cos(t * 3.141592653589793 / (12 * 3600.0));
    return 100 * (c > 0 ? c : 0.0);
}

}  // namespace obgc
