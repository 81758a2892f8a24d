"""ctypes wrapper of liboracle.so — TEST INFRASTRUCTURE, NOT THE PRODUCT.

The oracle is a CPU FP64 restatement of OceanBioME.jl's tracer-tendency path (see
obgc_oracle.h).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as
the oracle the GPU results are compared with.  It reuses only the parameter-struct mirrors of include/obgc.h.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from obgc import _abi as A

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "liboracle.so")
_lib = None

NUM_K = 13
K0, K1, K2, KB, KW, KS, KF, KP1, KP2, KP3, KSI, KSP_CALCITE, KSP_ARAGONITE = range(NUM_K)
NEWTON, NEWTON_SAFE, BISECTION, DAMPED = range(4)


class Model3D(C.Structure):
    _fields_ = [("npd", A.NPDParams), ("light", A.TwoBandParams), ("surface_kind", C.c_int32),
                ("advection", C.c_int32), ("surface_value", C.c_double), ("grid", A.Grid),
                ("n_tracers", C.c_int32), ("names", C.c_int32 * 32), ("negatives", C.c_int32),
                ("zero_exclude_mask", C.c_int32), ("invalid_fill_value", C.c_double),
                ("gas", C.POINTER(A.GasExchange) * 4), ("gas_target", C.c_int32 * 4), ("gas_dic", C.c_int32 * 4),
                ("gas_alk", C.c_int32 * 4), ("kappa_h", C.c_double),
                ("kappa_z_faces", C.POINTER(C.c_double)), ("vertical_implicit", C.c_int32),
                ("sed_receiver", C.c_int32), ("sed_sink_mask", C.c_uint32),
                ("sed_a", C.c_double), ("sed_b", C.c_double), ("sed_k", C.c_double),
                ("sed_storage", C.POINTER(C.c_double)), ("tendency_of", C.c_int32 * 32),
                ("forcing", C.POINTER(C.c_double) * 32), ("forcing_t0", C.c_double * 32), ("forcing_t1", C.c_double * 32),
                ("stage_rounding", C.c_double), ("rounding_seed", C.c_uint64), ("multig", C.c_void_p)]


class MultiG(C.Structure):
    _fields_ = [("p", A.MultiGParams), ("n_sinking", C.c_int32), ("sinking_slot", C.c_int32 * 4),
                ("no3", C.c_int32), ("nh4", C.c_int32), ("o2", C.c_int32),
                ("state", C.POINTER(C.c_double)), ("gcache", C.POINTER(C.c_double))]


class Pisces3D(C.Structure):
    _fields_ = [("p", A.PiscesParams), ("grid", A.Grid), ("nbands", C.c_int32), ("surface_kind", C.c_int32),
                ("kw", C.c_double * 4), ("e", C.c_double * 4), ("chi", C.c_double * 4), ("division", C.c_double * 4),
                ("surface_value", C.c_double), ("mixed_layer_depth", C.c_double), ("mean_kappa", C.c_double),
                ("advection", C.c_int32), ("negatives", C.c_int32), ("invalid_fill_value", C.c_double),
                ("carbon", A.CarbonOptions)]


NEG_NONE, NEG_SCALE, NEG_ZERO = 0, 1, 2
MAX_GROUPS, MAX_MEMBERS = 5, 10      # OR_MAX_GROUPS, OR_MAX_GROUP


class Column(C.Structure):
    _fields_ = [("Nz", C.c_int32), ("nsteps", C.c_int32), ("dz", C.c_double),
                ("surface_PAR", C.c_double), ("mu0", C.c_double), ("dt", C.c_double),
                ("pulse_step", C.c_int32), ("pulse_k", C.c_int32), ("pulse_amount", C.c_double),
                ("temperature", C.c_double), ("salinity", C.c_double)]


def build():
    """Compile liboracle.so with the Makefile beside this file (gcc, a few seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        P, D, I32, I64, VP = C.POINTER, C.c_double, C.c_int32, C.c_int64, C.c_void_p
        L.or_npd_preset.argtypes = [C.c_int, P(A.NPDParams)]
        L.or_npd_required_tracers.argtypes = [P(A.NPDParams), P(I32), C.c_int]
        L.or_npd_tendency.argtypes = [P(A.NPDParams), C.c_int, P(D), D]
        L.or_npd_tendency.restype = D
        L.or_npd_drift_profile.argtypes = [P(A.NPDParams), C.c_int, C.c_int, P(D), P(C.c_int)]
        L.or_twoband_column.argtypes = [P(A.TwoBandParams), C.c_int, P(D), P(D), P(D), D, P(D)]
        L.or_multiband_column.argtypes = [C.c_int, P(D), D, D, D, P(D), D, P(D)]
        L.or_euphotic_depth_column.argtypes = [C.c_int, P(D), P(D), D, D]
        L.or_euphotic_depth_column.restype = D
        L.or_multiband_coefficients.argtypes = [C.c_int, P(D), C.c_int, P(D), P(D), P(D), P(D), P(D), P(D), P(D)]
        L.or_default_surface_PAR.argtypes = [D]
        L.or_default_surface_PAR.restype = D
        L.or_equilibrium_constant.argtypes = [C.c_int, D, D, C.c_int, D]
        L.or_equilibrium_constant.restype = D
        L.or_pressure_correction.argtypes = [C.c_int, D, D]
        L.or_pressure_correction.restype = D
        L.or_first_virial.argtypes = [D]
        L.or_first_virial.restype = D
        L.or_cross_virial.argtypes = [D]
        L.or_cross_virial.restype = D
        L.or_density_eos80.argtypes = [D, D, D]
        L.or_density_eos80.restype = D
        L.or_density_teos10_polynomial.argtypes = [D, D, D]
        L.or_density_teos10_polynomial.restype = D
        L.or_carbon_default_options.argtypes = [P(A.CarbonOptions)]
        L.or_carbon_chemistry.argtypes = [P(A.CarbonOptions), D, D, D, D, D, D, D, D, P(D), P(C.c_int)]
        L.or_carbon_chemistry_batch.argtypes = [P(A.CarbonOptions), I64, P(D), P(D), P(D), P(D),
                                                VP, VP, VP, VP, P(D), C.c_int]
        L.or_solve_test_function.argtypes = [C.c_int, C.c_int, D, D, D, D, D]
        L.or_solve_test_function.restype = D
        L.or_box_run.argtypes = [P(A.NPDParams), P(D), VP, D, D, D, C.c_int]
        L.or_box_run_drivers.argtypes = [P(A.NPDParams), P(D), VP, D, D, C.c_int, C.c_int, P(I32), P(P(D)), C.c_int,
                                         P(I32), P(P(D))]
        L.or_step3d.argtypes = [P(Model3D), P(D), VP, VP, VP, D, D, C.c_int, C.c_int]
        L.or_stage3d.argtypes = [P(Model3D), P(D), VP, VP, VP, D, D, C.c_int, P(D), P(D), VP, C.c_int]
        L.or_par3d.argtypes = [P(Model3D), P(D), D, P(D), C.c_int]
        L.or_columns_run.argtypes = [P(A.NPDParams), P(A.TwoBandParams), C.c_int, P(Column), P(I64),
                                     P(I64), C.c_int, P(I32), P(D), P(D), D, D, C.c_int, C.c_int, D, C.c_int,
                                     P(A.GasExchange)]
        L.or_scale_negatives.argtypes = [I64, C.c_int, P(P(D)), P(D), D]
        L.or_pisces_defaults.argtypes = [P(A.PiscesParams)]
        L.or_cbm_day_length.argtypes = [D, D, D]
        L.or_cbm_day_length.restype = D
        L.or_pisces_tendency.argtypes = [P(A.PiscesParams), C.c_int, P(D), P(D), D, D]
        L.or_pisces_tendency.restype = D
        L.or_pisces_tendencies.argtypes = [P(A.PiscesParams), P(D), P(D), D, D, P(D)]
        L.or_pisces_goc_speed.argtypes = [P(A.PiscesParams), C.c_int, P(D), D, D, P(D)]
        L.or_mixed_layer_mean.argtypes = [C.c_int, P(D), P(D), D]
        L.or_mixed_layer_mean.restype = D
        L.or_pisces_conserved_groups.argtypes = [P(A.PiscesParams), P(I32), P(I32), P(D)]
        L.or_gas_exchange_defaults.argtypes = [C.c_int, P(A.GasExchange)]
        L.or_schmidt_number.argtypes = [P(D), D]
        L.or_schmidt_number.restype = D
        L.or_transfer_velocity_660.argtypes = [P(D), D]
        L.or_transfer_velocity_660.restype = D
        L.or_o2_solubility.argtypes = [P(D), D, D]
        L.or_o2_solubility.restype = D
        L.or_gas_exchange_flux.argtypes = [P(A.GasExchange), D, D, D, D, D, D, D]
        L.or_gas_exchange_flux.restype = D
        L.or_pisces_step3d.argtypes = [P(Pisces3D), P(D), VP, VP, D, D, C.c_int, C.c_int]
        L.or_pisces_stage3d.argtypes = [P(Pisces3D), P(D), VP, VP, D, D, C.c_int, P(D), P(D), C.c_int, C.c_int]
        L.or_pisces_update_state3d.argtypes = [P(Pisces3D), P(D), D, P(D), P(D), P(D), C.c_int]
        L.or_conserved_groups.argtypes = [P(A.NPDParams), C.c_int, P(I32), P(I32), P(I32), P(D)]
        L.or_scale_cell.argtypes = [P(D), C.c_long, C.c_int, P(I32), P(I32), P(D), D]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _opt(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def nthreads():
    return os.cpu_count() or 1


# ---------------------------------------------------------------------------- NPD
def preset(name):
    p = A.NPDParams()
    lib().or_npd_preset({"LOBSTER": A.PRESET_LOBSTER, "NPZD": A.PRESET_NPZD}[name], C.byref(p))
    return p


def required_tracers(p):
    buf = (C.c_int32 * 32)()
    n = lib().or_npd_required_tracers(C.byref(p), buf, 32)
    return [buf[i] for i in range(n)]


def tendency(p, name, values, PAR):
    v = np.zeros(A.NUM_NAMED)
    for k, x in values.items():
        v[A.NAME_INDEX[k] if isinstance(k, str) else k] = x
    idx = A.NAME_INDEX[name] if isinstance(name, str) else name
    return lib().or_npd_tendency(C.byref(p), idx, _dp(v), PAR)


def tendencies_array(p, vals, PAR):
    """vals: (n, NUM_NAMED) array, PAR (n,) -> (n, NUM_NAMED) tendencies (0 where not required)."""
    out = np.zeros_like(vals)
    names = required_tracers(p)
    L = lib()
    for c in range(vals.shape[0]):
        row = np.ascontiguousarray(vals[c])
        for nm in names:
            out[c, nm] = L.or_npd_tendency(C.byref(p), nm, _dp(row), float(PAR[c]))
    return out


def drift_profile(p, name, Nz):
    w = np.zeros(Nz + 1)
    d = C.c_int(0)
    lib().or_npd_drift_profile(C.byref(p), A.NAME_INDEX[name] if isinstance(name, str) else name, Nz, _dp(w), C.byref(d))
    return w if d.value else None


# ---------------------------------------------------------------------------- light
def twoband_column(lp, zc, zf, P, PAR0):
    zc, zf, P = (np.ascontiguousarray(x, dtype=np.float64) for x in (zc, zf, P))
    out = np.zeros(len(zc))
    lib().or_twoband_column(C.byref(lp), len(zc), _dp(zc), _dp(zf), _dp(P), PAR0, _dp(out))
    return out


def multiband_column(zc, kw, e, chi, Chl, surface):
    zc, Chl = (np.ascontiguousarray(x, dtype=np.float64) for x in (zc, Chl))
    out = np.zeros(len(zc))
    lib().or_multiband_column(len(zc), _dp(zc), kw, e, chi, _dp(Chl), surface, _dp(out))
    return out


def multiband_coefficients(bands, lam, kw, e, chi):
    edges = np.array([x for b in bands for x in b], dtype=np.float64)
    lam, kw, e, chi = (np.ascontiguousarray(x, dtype=np.float64) for x in (lam, kw, e, chi))
    n = len(bands)
    okw, oe, ochi = np.zeros(n), np.zeros(n), np.zeros(n)
    lib().or_multiband_coefficients(n, _dp(edges), len(lam), _dp(lam), _dp(kw), _dp(e), _dp(chi),
                                    _dp(okw), _dp(oe), _dp(ochi))
    return okw, oe, ochi


def euphotic_depth_column(zc_with_halo, PAR, PAR_top_halo, cutoff=1e-3):
    zc, PAR = (np.ascontiguousarray(x, dtype=np.float64) for x in (zc_with_halo, PAR))
    return lib().or_euphotic_depth_column(len(PAR), _dp(zc), _dp(PAR), PAR_top_halo, cutoff)


def default_surface_PAR(t):
    return lib().or_default_surface_PAR(t)


# ---------------------------------------------------------------------------- carbon
def K(which, Tk, S, P=None):
    return lib().or_equilibrium_constant(which, Tk, S, 0 if P is None else 1, 0.0 if P is None else P)


def pressure_correction(which, Tk, P):
    return lib().or_pressure_correction(which, Tk, P)


def density_eos80(T, S, P):
    return lib().or_density_eos80(T, S, P)


def density_teos10_polynomial(T, S, P):
    return lib().or_density_teos10_polynomial(T, S, P)


def carbon_options(**kw):
    o = A.CarbonOptions()
    lib().or_carbon_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def carbon_chemistry(DIC, T, S, Alk=0.0, pH=None, P=None, silicate=0.0, phosphate=0.0,
                     output=A.OUT_FCO2, density=None, return_iters=False, **kw):
    o = carbon_options(output=output, **kw)
    if density == "eos80":
        o.density = A.DENSITY_EOS80
    elif density is not None:
        o.density, o.density_value = A.DENSITY_CONSTANT, density
    if pH is not None:
        o.ph_given = 1
    if P is not None:
        o.has_pressure = 1
    out = C.c_double(0)
    it = C.c_int(0)
    lib().or_carbon_chemistry(C.byref(o), DIC, Alk, T, S, silicate, phosphate,
                              0.0 if P is None else P, 0.0 if pH is None else pH, C.byref(out), C.byref(it))
    return (out.value, it.value) if return_iters else out.value


def carbon_chemistry_batch(o, DIC, Alk, T, S, Si=None, PO4=None, P=None, pH=None, threads=None):
    arrs = [np.ascontiguousarray(x, dtype=np.float64) if x is not None else None
            for x in (DIC, Alk, T, S, Si, PO4, P, pH)]
    n = len(arrs[0])
    out = np.zeros(n)
    lib().or_carbon_chemistry_batch(C.byref(o), n, _dp(arrs[0]), _dp(arrs[1]), _dp(arrs[2]), _dp(arrs[3]),
                                    _opt(arrs[4]), _opt(arrs[5]), _opt(arrs[6]), _opt(arrs[7]), _dp(out),
                                    threads or nthreads())
    return out


def solve(solver, fid, x0, x1=0.0, damping=0.5, pa=1.0, pb=-2.0):
    return lib().or_solve_test_function(solver, fid, float(x0), float(x1), damping, pa, pb)


# ---------------------------------------------------------------------------- stepping
def box_run(p, values, dt, nsteps, PAR_stages=None, PAR_const=0.0, t0=0.0):
    v = np.zeros(A.NUM_NAMED)
    for k, x in values.items():
        v[A.NAME_INDEX[k] if isinstance(k, str) else k] = x
    ps = None if PAR_stages is None else np.ascontiguousarray(PAR_stages, dtype=np.float64)
    lib().or_box_run(C.byref(p), _dp(v), _opt(ps), PAR_const, t0, dt, nsteps)
    return v


def box_run_drivers(p, values, dt, nsteps, PAR_stages=None, PAR_const=0.0, prescribed=None, forcing=None):
    """prescribed={name: values [3 nsteps + 1]}, forcing={name: rates [3 nsteps]} at the stage times."""
    v = np.zeros(A.NUM_NAMED)
    for k, x in values.items():
        v[A.NAME_INDEX[k] if isinstance(k, str) else k] = x
    ps = None if PAR_stages is None else np.ascontiguousarray(PAR_stages, dtype=np.float64)
    pres = [(A.NAME_INDEX[k], np.ascontiguousarray(a, dtype=np.float64)) for k, a in (prescribed or {}).items()]
    frcs = [(A.NAME_INDEX[k], np.ascontiguousarray(a, dtype=np.float64)) for k, a in (forcing or {}).items()]
    pn = (C.c_int32 * max(1, len(pres)))(*[q for q, _ in pres])
    pp = (C.POINTER(C.c_double) * max(1, len(pres)))(*[_dp(a) for _, a in pres])
    fn = (C.c_int32 * max(1, len(frcs)))(*[q for q, _ in frcs])
    fp = (C.POINTER(C.c_double) * max(1, len(frcs)))(*[_dp(a) for _, a in frcs])
    lib().or_box_run_drivers(C.byref(p), _dp(v), _opt(ps), PAR_const, dt, nsteps, len(pres), pn, pp, len(frcs), fn, fp)
    return v


def model3d(p, grid, names, light=None, surface_kind=A.SURFACE_DEFAULT, surface_value=0.0, advection=1,
            negatives=NEG_NONE, zero_exclude=(), invalid_fill_value=float("nan"), gas_exchange=(), kappa_h=0.0,
            kappa_z_faces=None, sediment=None, tendency_of=None, forcing=None, vertical_implicit=False):
    """gas_exchange: top boundary conditions, each an A.GasExchange struct (CO2 on DIC with DIC and
    Alk, O2 on O2) or a tuple (struct, target, dic, alk) of tracer names or slots (None for passive
    entries of `names`); kappa_h, kappa_z_faces[Nz + 1]: ScalarDiffusivity (explicit).
    sediment=(sinking names, receiver, a, b, k, storage array [Ny, Nx] float64) for
    InstantRemineralisation.  tendency_of={slot: "DIC" | "Alk"}: passive slots taking that BGC
    tendency (CarbonateSystem replicates).  forcing={slot: (rate array [Nz, Ny, Nx], t0, t1)}."""
    m = Model3D()
    nm_all = [-1 if n is None else (A.NAME_INDEX[n] if isinstance(n, str) else n) for n in names]

    def slot(x):   # a slot index, or a tracer name
        return x if isinstance(x, int) else nm_all.index(A.NAME_INDEX[x])
    m._gas_keep = []
    for q, g in enumerate(gas_exchange):
        if not isinstance(g, tuple):
            g = (g, "DIC", "DIC", "Alk") if g.gas == A.GAS_CO2 else (g, "O2", None, None)
        ge, target, dic, alk = g
        m._gas_keep.append(ge)
        m.gas[q] = C.pointer(ge)
        m.gas_target[q] = slot(target)
        m.gas_dic[q] = slot(dic) if dic is not None else -1
        m.gas_alk[q] = slot(alk) if alk is not None else -1
    for q, src in (tendency_of or {}).items():
        m.tendency_of[q] = A.NAME_INDEX[src] + 1
    m._forcing_keep = []
    for q, (rate, t0, t1) in (forcing or {}).items():
        r = np.ascontiguousarray(rate, dtype=np.float64)
        m._forcing_keep.append(r)
        m.forcing[q] = r.ctypes.data_as(C.POINTER(C.c_double))
        m.forcing_t0[q], m.forcing_t1[q] = t0, t1
    m.sed_receiver = -1
    if sediment is not None:
        sinking, receiver, sa, sb, sk, storage = sediment
        nm = [A.NAME_INDEX[n] if isinstance(n, str) else n for n in names]
        m.sed_receiver = nm.index(A.NAME_INDEX[receiver])
        m.sed_sink_mask = sum(1 << nm.index(A.NAME_INDEX[n]) for n in sinking)
        m.sed_a, m.sed_b, m.sed_k = sa, sb, sk
        assert storage.dtype == np.float64 and storage.flags.c_contiguous
        m._storage = storage
        m.sed_storage = storage.ctypes.data_as(C.POINTER(C.c_double))
    m.kappa_h = kappa_h
    m.vertical_implicit = int(bool(vertical_implicit))
    if kappa_z_faces is not None:
        m._kz = np.ascontiguousarray(kappa_z_faces, dtype=np.float64)
        m.kappa_z_faces = m._kz.ctypes.data_as(C.POINTER(C.c_double))
    m.negatives = negatives
    m.invalid_fill_value = invalid_fill_value
    m.zero_exclude_mask = sum(1 << q for q, nm in enumerate(names) if nm in zero_exclude)
    m.npd = p
    m.light = light if light is not None else A.default_twoband()
    m.surface_kind = surface_kind
    m.surface_value = surface_value
    m.advection = advection
    m.grid = grid
    m.n_tracers = len(names)
    for q, nm in enumerate(names):
        m.names[q] = -1 if nm is None else (A.NAME_INDEX[nm] if isinstance(nm, str) else nm)
    return m


def attach_multig(m, params, names, sinking, grid, state=None):
    """Give model `m` a SimpleMultiG sediment: params (A.MultiGParams; sedimentation_rate <= 0 is
    resolved from the grid's bottom cell), tracer names of the model's slots, the sinking tracers.
    Returns the sediment's field array [4][Ny*Nx] (Ns, Nf, Nr, started), updated in place by step3d."""
    mg = MultiG()
    C.memmove(C.byref(mg.p), C.byref(params), C.sizeof(A.MultiGParams))
    if not (mg.p.sedimentation_rate > 0):
        zb = -grid.Lz + 0.5 * grid.Lz / grid.Nz
        mg.p.sedimentation_rate = 982.0 * abs(zb) ** -1.548
    idx = {n: q for q, n in enumerate(names)}
    mg.n_sinking = len(sinking)
    for q, n in enumerate(sinking):
        mg.sinking_slot[q] = idx[n]
    mg.no3, mg.nh4, mg.o2 = idx["NO3"], idx["NH4"], idx["O2"]
    NN = grid.Nx * grid.Ny
    st = np.zeros(4 * NN) if state is None else np.ascontiguousarray(state, dtype=np.float64)
    gc = np.zeros(3 * NN)
    mg.state = st.ctypes.data_as(C.POINTER(C.c_double))
    mg.gcache = gc.ctypes.data_as(C.POINTER(C.c_double))
    m._mg_keep = (mg, st, gc)
    m.multig = C.cast(C.pointer(mg), C.c_void_p)
    return st


def step3d(m, state, u=None, v=None, w=None, t=0.0, dt=1.0, nsteps=1, threads=None):
    """state: float64 array (n_tracers, Nz, Ny, Nx), stepped in place."""
    assert state.dtype == np.float64 and state.flags.c_contiguous
    lib().or_step3d(C.byref(m), _dp(state), _opt(u), _opt(v), _opt(w), t, dt, nsteps, threads or nthreads())
    return state


def stage3d(m, state, G, Gm, u=None, v=None, w=None, t=0.0, dt=1.0, stage=0, sed_Gm=None, threads=None):
    """One RK3 stage in place (or_stage3d): G receives the stage's tendency, Gm holds the previous
    stage's; swap them before the next stage."""
    for a in (state, G, Gm):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    lib().or_stage3d(C.byref(m), _dp(state), _opt(u), _opt(v), _opt(w), t, dt, stage, _dp(G), _dp(Gm), _opt(sed_Gm),
                     threads or nthreads())
    return state


def par3d(m, state, t, threads=None):
    g = m.grid
    out = np.zeros((g.Nz, g.Ny, g.Nx))
    lib().or_par3d(C.byref(m), _dp(state), t, _dp(out), threads or nthreads())
    return out


def conserved_groups(p, names):
    """or_conserved_groups: [(slots, factors), ...] in the reference's group and member order."""
    nm = np.array([A.NAME_INDEX[x] if isinstance(x, str) else x for x in names], dtype=np.int32)
    gn = (C.c_int32 * MAX_GROUPS)()
    gs = (C.c_int32 * (MAX_GROUPS * MAX_MEMBERS))()
    gf = (C.c_double * (MAX_GROUPS * MAX_MEMBERS))()
    ng = lib().or_conserved_groups(C.byref(p), len(nm), nm.ctypes.data_as(C.POINTER(C.c_int32)), gn, gs, gf)
    return _groups(ng, gn, gs, gf)


def _groups(ng, gn, gs, gf):
    return [([gs[g * MAX_MEMBERS + m] for m in range(gn[g])], [gf[g * MAX_MEMBERS + m] for m in range(gn[g])])
            for g in range(ng)]


def group_arrays(groups):
    """(gn, gslot, gfac) arrays in or_scale_cell's layout for a list of (slots, factors)."""
    gn = np.array([len(g[0]) for g in groups], dtype=np.int32)
    gs = np.zeros(MAX_GROUPS * MAX_MEMBERS, dtype=np.int32)
    gf = np.zeros(MAX_GROUPS * MAX_MEMBERS)
    for g, (sl, fa) in enumerate(groups):
        gs[g * MAX_MEMBERS:g * MAX_MEMBERS + len(sl)] = sl
        gf[g * MAX_MEMBERS:g * MAX_MEMBERS + len(fa)] = fa
    return gn, gs, gf


def columns_run(p, lp, cols, names, state, kappa, state_offsets, kappa_offsets, dt, nsteps, threads=None,
                negatives=NEG_NONE, invalid_fill_value=float("nan"), gas=None):
    """gas: an A.GasExchange (CO2) as the top boundary condition of DIC, or None."""
    n = len(cols)
    carr = (Column * n)(*cols)
    so = np.ascontiguousarray(state_offsets, dtype=np.int64)
    ko = np.ascontiguousarray(kappa_offsets, dtype=np.int64)
    nm = np.array([A.NAME_INDEX[x] if isinstance(x, str) else x for x in names], dtype=np.int32)
    lib().or_columns_run(C.byref(p), C.byref(lp), n, carr, so.ctypes.data_as(C.POINTER(C.c_int64)),
                         ko.ctypes.data_as(C.POINTER(C.c_int64)), len(names),
                         nm.ctypes.data_as(C.POINTER(C.c_int32)), _dp(state), _dp(kappa), 0.0, dt,
                         nsteps, negatives, invalid_fill_value, threads or nthreads(),
                         None if gas is None else C.byref(gas))
    return state


def scale_negatives(fields, scalefactors, fill=np.nan):
    ptrs = (C.POINTER(C.c_double) * len(fields))(*[_dp(f) for f in fields])
    sf = np.ascontiguousarray(scalefactors, dtype=np.float64)
    lib().or_scale_negatives(len(fields[0]), len(fields), ptrs, _dp(sf), fill)


# ----------------------------------------------------------------------------- PISCES
def pisces_defaults():
    p = A.PiscesParams()
    lib().or_pisces_defaults(C.byref(p))
    return p


def pisces_tendencies(p, values, aux, z, t=0.0):
    """values: 26 tracer values (PISCES order or a dict by name), aux: 12 auxiliary values or a dict."""
    if isinstance(values, dict):
        values = [float(values.get(n, values.get(a, 0.0))) for n, a in zip(A.PISCES_TRACERS, A.PISCES_ASCII)]
    if isinstance(aux, dict):
        aux = [float(aux[n]) for n in A.PISCES_AUX]
    v = np.ascontiguousarray(values, dtype=np.float64)
    a = np.ascontiguousarray(aux, dtype=np.float64)
    G = np.zeros(A.PISCES_NUM_BGC)
    lib().or_pisces_tendencies(C.byref(p), _dp(v), _dp(a), float(z), float(t), _dp(G))
    return G


def pisces_conserved_groups(p):
    gn = (C.c_int32 * MAX_GROUPS)()
    gs = (C.c_int32 * (MAX_GROUPS * MAX_MEMBERS))()
    gf = (C.c_double * (MAX_GROUPS * MAX_MEMBERS))()
    ng = lib().or_pisces_conserved_groups(C.byref(p), gn, gs, gf)
    return _groups(ng, gn, gs, gf)


def mixed_layer_mean(zf, C_, zmxl):
    zf = np.ascontiguousarray(zf, dtype=np.float64)
    C_ = np.ascontiguousarray(C_, dtype=np.float64)
    return lib().or_mixed_layer_mean(len(C_), _dp(zf), _dp(C_), float(zmxl))


def goc_speed(p, zc, zmxl, zeu):
    zc = np.ascontiguousarray(zc, dtype=np.float64)
    w = np.zeros(len(zc) + 1)
    lib().or_pisces_goc_speed(C.byref(p), len(zc), _dp(zc), float(zmxl), float(zeu), _dp(w))
    return w


def pisces3d(p, grid, light, mixed_layer_depth, mean_kappa=1.0, surface_kind=A.SURFACE_DEFAULT, surface_value=0.0,
             advection=1, negatives=NEG_NONE, invalid_fill_value=float("nan")):
    m = Pisces3D()
    m.p = p
    m.grid = grid
    m.nbands = len(light.kw)
    m.surface_kind = surface_kind
    for b in range(m.nbands):
        m.kw[b], m.e[b], m.chi[b], m.division[b] = light.kw[b], light.e[b], light.chi[b], light.division[b]
    m.surface_value = surface_value
    m.mixed_layer_depth = mixed_layer_depth
    m.mean_kappa = mean_kappa
    m.advection = advection
    m.negatives = negatives
    m.invalid_fill_value = invalid_fill_value
    m.carbon = carbon_options()
    return m


def pisces_step3d(m, state, u=None, v=None, t=0.0, dt=1.0, nsteps=1, threads=None):
    """state: float64 (26, Nz, Ny, Nx), stepped in place."""
    assert state.dtype == np.float64 and state.flags.c_contiguous
    lib().or_pisces_step3d(C.byref(m), _dp(state), _opt(u), _opt(v), t, dt, nsteps, threads or nthreads())
    return state


def pisces_stage3d(m, state, G, Gm, u=None, v=None, t=0.0, dt=1.0, stage=0, start=False, threads=None):
    """One RK3 stage in place (or_pisces_stage3d): G receives the stage's tendency, Gm holds the
    previous stage's; swap them before the next stage.  start: the modifier first, as
    pisces_step3d applies it on entry."""
    for a in (state, G, Gm):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    lib().or_pisces_stage3d(C.byref(m), _dp(state), _opt(u), _opt(v), t, dt, stage, _dp(G), _dp(Gm), int(bool(start)),
                            threads or nthreads())
    return state


def pisces_update_state3d(m, state, t, threads=None):
    g = m.grid
    N = g.Nx * g.Ny * g.Nz
    par4 = np.zeros(4 * N)
    xy2 = np.zeros(2 * g.Nx * g.Ny)
    omega = np.zeros(N)
    lib().or_pisces_update_state3d(C.byref(m), _dp(np.ascontiguousarray(state, dtype=np.float64)), t, _dp(par4),
                                   _dp(xy2), _dp(omega), threads or nthreads())
    shp = (g.Nz, g.Ny, g.Nx)
    return par4.reshape((4,) + shp), xy2.reshape(2, g.Ny, g.Nx), omega.reshape(shp)


def gas_exchange_defaults(gas):
    g = A.GasExchange()
    assert lib().or_gas_exchange_defaults(gas, C.byref(g)) == 0
    return g


def schmidt_number(g, T):
    return lib().or_schmidt_number(g.schmidt, T)


def o2_solubility(g, T, S):
    return lib().or_o2_solubility(g.o2_solubility, T, S)


def gas_exchange_flux(g, T, S, DIC=0.0, Alk=0.0, O2=0.0, u10=None, air=None):
    return lib().or_gas_exchange_flux(C.byref(g), T, S, DIC, Alk, O2, g.wind_speed if u10 is None else u10,
                                      g.air_concentration if air is None else air)

