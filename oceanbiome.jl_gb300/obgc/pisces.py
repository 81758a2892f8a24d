"""PISCES mirror (src/Models/AdvectedPopulations/PISCES): parameters, the per-cell tendencies of all
24 tracers on the GPU, and the update_biogeochemical_state! pieces (mixed-layer means, calcite
saturation).  Tracers follow required_biogeochemical_tracers(::PISCES) (PISCES.jl:86-98)."""
import ctypes as C
import math

import numpy as np

from . import _abi as A


class PISCES:
    """PISCES(; grid, ...overrides): holds the C parameter struct with the reference's defaults.
    Nested components are reached by attribute path, e.g. PISCES(grid, **{"nano.dark_tolerance": 2 * 86400})."""

    def __init__(self, grid=None, scale_negatives=False, invalid_fill_value=math.nan, **overrides):
        self.grid = grid
        self.params = A.PiscesParams()
        A.check(A.load().obgc_pisces_default_params(C.byref(self.params)), "obgc_pisces_default_params")
        for path, value in overrides.items():
            obj = self.params
            parts = path.split(".")
            for part in parts[:-1]:
                obj = getattr(obj, part)
            if not hasattr(obj, parts[-1]):
                raise ValueError(f"PISCES has no parameter {path!r}")
            setattr(obj, parts[-1], value)
        self.scale_negatives = scale_negatives
        self.invalid_fill_value = invalid_fill_value

    def __repr__(self):
        return "PISCES (" + ", ".join(A.PISCES_TRACERS) + ")"


def required_biogeochemical_tracers(_bgc=None):
    return tuple(A.PISCES_TRACERS)


def required_biogeochemical_auxiliary_fields(_bgc=None):
    """PISCES.jl:100-101 (zₘₓₗ, zₑᵤ, Si′, Ω, κ, mixed_layer_PAR, wPOC, wGOC, PAR, PAR₁, PAR₂, PAR₃)."""
    return tuple(A.PISCES_AUX)


def _by_name(d, q):
    """Entry q of the PISCES tracer order, keyed by the reference's name (NO₃) or its ASCII form (NO3)."""
    return d[A.PISCES_TRACERS[q]] if A.PISCES_TRACERS[q] in d else d[A.PISCES_ASCII[q]]


def _field(x, grid, torch):
    f = A.PiscesField()
    if x is None or x == "auto":
        f.kind = A.PF_AUTO
    elif isinstance(x, (int, float)):
        f.kind, f.value = A.PF_CONSTANT, float(x)
    else:
        shp = tuple(x.shape)
        if shp == (grid.Ny, grid.Nx):
            f.kind = A.PF_XY
        elif shp == (grid.Nz + 1, grid.Ny, grid.Nx):
            f.kind = A.PF_ZFACE
        elif shp == grid.shape:
            f.kind = A.PF_XYZ
        else:
            raise ValueError(f"auxiliary field of shape {shp} fits none of (Ny, Nx), (Nz, Ny, Nx), (Nz+1, Ny, Nx)")
        f.data = x.data_ptr()
    return f


def pisces_tendencies(bgc, grid, tracers, aux, G, t=0.0, stream=0):
    """tracers: dict name -> device tensor (Nz, Ny, Nx) for all 26 tracers; aux: dict of the 12
    auxiliary inputs (number, (Ny, Nx) or (Nz[+1], Ny, Nx) tensor, or "auto" for wPOC / wGOC);
    G: dict name -> output tensor for the 24 tracers with tendencies."""
    import torch
    dt = A.F32 if _by_name(tracers, 0).dtype == torch.float32 else A.F64
    tr = (C.c_void_p * 26)(*[_by_name(tracers, q).data_ptr() for q in range(26)])
    gs = (C.c_void_p * 24)(*[_by_name(G, q).data_ptr() for q in range(24)])
    ax = (A.PiscesField * 12)(*[_field(aux.get(n), grid, torch) for n in A.PISCES_AUX])
    A.check(A.load().obgc_pisces_tendencies(C.byref(bgc.params), C.byref(grid.c_grid()), dt, tr, ax, gs, float(t),
                                            C.c_void_p(stream)), "obgc_pisces_tendencies")


def mixed_layer_mean(grid, field, mixed_layer_depth, out, stream=0):
    """compute_mixed_layer_mean! (mean_mixed_layer_properties.jl:10-46) into out (Ny, Nx)."""
    import torch
    dt = A.F32 if field.dtype == torch.float32 else A.F64
    z = _field(mixed_layer_depth, grid, torch)
    A.check(A.load().obgc_mixed_layer_mean(C.byref(grid.c_grid()), dt, field.data_ptr(), C.byref(z), out.data_ptr(),
                                           C.c_void_p(stream)), "obgc_mixed_layer_mean")
    return out


def calcite_saturation(grid, DIC, Alk, T, S, Si, out, carbon_chemistry=None, stream=0):
    """compute_calcite_saturation! (compute_calcite_saturation.jl:9-37) into out (Nz, Ny, Nx)."""
    import torch
    from .carbon import CarbonChemistry
    cc = carbon_chemistry or CarbonChemistry()
    dt = A.F32 if DIC.dtype == torch.float32 else A.F64
    A.check(A.load().obgc_pisces_calcite_saturation(C.byref(cc.options), C.byref(grid.c_grid()), dt, DIC.data_ptr(),
                                                    Alk.data_ptr(), T.data_ptr(), S.data_ptr(),
                                                    None if Si is None else Si.data_ptr(), out.data_ptr(),
                                                    C.c_void_p(stream)), "obgc_pisces_calcite_saturation")
    return out


class _Tracers(dict):
    """model.tracers: keyed by the reference's names (NO₃), also reachable by their ASCII forms (NO3)."""

    def __getitem__(self, name):
        return dict.__getitem__(self, A.PISCES_TRACERS[A.PISCES_INDEX[name]])

    def __contains__(self, name):
        return name in A.PISCES_INDEX


class PiscesModel:
    """A 3-D PISCES model on the device: NonhydrostaticModel(grid; biogeochemistry = PISCES(...))
    with MultiBand light (3 bands), a prescribed uniform mixed-layer depth, prescribed velocities and
    WENO5 advection; time_step runs update_biogeochemical_state! and the fused RK3 substeps."""

    def __init__(self, grid, biogeochemistry=None, velocities=None, precision="f32", mixed_layer_depth=-50.0,
                 mean_kappa=1.0, surface_PAR=None, light=None, advection=True, device="cuda"):
        import torch
        from .light import MultiBandPhotosyntheticallyActiveRadiation
        from .carbon import CarbonChemistry
        self.grid = grid
        self.bgc = bgc = biogeochemistry or PISCES(grid)
        self.precision = precision
        self.dtype = torch.float32 if precision == "f32" else torch.float64
        self.light = light or MultiBandPhotosyntheticallyActiveRadiation(grid=grid, surface_PAR=surface_PAR)
        d = A.PiscesModelDesc()
        d.pisces = bgc.params
        d.grid = grid.c_grid()
        d.precision = {"f32": A.PREC_F32, "mixed": A.PREC_MIXED, "f64": A.PREC_F64}[precision]
        d.advection = A.ADVECTION_WENO5 if advection else A.ADVECTION_NONE
        d.nbands = len(self.light.kw)
        d.negatives = A.NEGATIVES_SCALE if bgc.scale_negatives else A.NEGATIVES_NONE
        for b in range(d.nbands):
            d.kw[b], d.e[b], d.chi[b], d.division[b] = self.light.kw[b], self.light.e[b], self.light.chi[b], self.light.division[b]
        d.surface = self.light.surface
        d.mixed_layer_depth = float(mixed_layer_depth)
        d.mean_kappa = float(mean_kappa)
        d.invalid_fill_value = float(bgc.invalid_fill_value)
        d.carbon = CarbonChemistry().options
        self.desc = d
        self._lib = lib = A.load()
        h = C.c_void_p()
        A.check(lib.obgc_pisces_model_create(C.byref(d), C.byref(h)), "obgc_pisces_model_create")
        self._h = h
        self.tracers = _Tracers((n, torch.zeros(grid.shape, dtype=self.dtype, device=device)) for n in A.PISCES_TRACERS)
        u, v = (velocities or (None, None))[:2]
        self.velocities = tuple(None if x is None else x.to(device=device, dtype=self.dtype).contiguous() for x in (u, v))
        ptrs = (C.c_void_p * 26)(*[self.tracers[n].data_ptr() for n in A.PISCES_TRACERS])
        A.check(lib.obgc_pisces_model_bind(h, ptrs, *(None if x is None else x.data_ptr() for x in self.velocities)),
                "obgc_pisces_model_bind")
        self.time = 0.0

    def close(self):
        if self._h:
            self._lib.obgc_pisces_model_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_(self, **values):
        import torch
        for k, v in values.items():
            name = A.PISCES_TRACERS[A.PISCES_INDEX[k]]
            self.tracers[name].copy_(torch.as_tensor(v, dtype=self.dtype).expand(self.grid.shape))

    def state_array(self):
        import torch
        return torch.stack([self.tracers[n] for n in A.PISCES_TRACERS])

    def update_state(self, t=None, stream=0):
        A.check(self._lib.obgc_pisces_model_update_state(self._h, float(self.time if t is None else t), C.c_void_p(stream)),
                "obgc_pisces_model_update_state")

    def time_step(self, dt, nsteps=1, stream=0):
        A.check(self._lib.obgc_pisces_model_step(self._h, float(self.time), float(dt), int(nsteps), C.c_void_p(stream)),
                "obgc_pisces_model_step")
        self.time += dt * nsteps

    def field(self, which):
        """"PAR", "PAR1".."PAR3", "zeu", "mixed_layer_PAR", "Omega": a host FP64 copy of the model's buffer."""
        idx = {"PAR": 0, "PAR1": 1, "PAR2": 2, "PAR3": 3, "zeu": 4, "mixed_layer_PAR": 5, "Omega": 6}[which]
        shape = (self.grid.Ny, self.grid.Nx) if idx in (4, 5) else self.grid.shape
        out = np.empty(shape, dtype=np.float64)
        A.check(self._lib.obgc_pisces_model_read_field(self._h, idx, out.ctypes.data_as(C.POINTER(C.c_double))),
                "obgc_pisces_model_read_field")
        return out

    def set_profiling(self, on=True):
        A.check(self._lib.obgc_pisces_model_set_profiling(self._h, int(bool(on))), "obgc_pisces_model_set_profiling")

    def last_timing(self):
        """Device ms of the last profiled time_step, summed over its RK3 stages, by phase."""
        ms = (C.c_double * 4)()
        n = C.c_int32()
        A.check(self._lib.obgc_pisces_model_last_timing(self._h, ms, C.byref(n)), "obgc_pisces_model_last_timing")
        return dict(light=ms[0], calcite=ms[1], functor=ms[2], substep=ms[3], stages=n.value)

