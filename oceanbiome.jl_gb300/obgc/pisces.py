"""PISCES mirror (src/Models/AdvectedPopulations/PISCES): parameters, the per-cell tendencies of all
24 tracers on the GPU, and the update_biogeochemical_state! pieces (mixed-layer means, calcite
saturation).  Tracers follow required_biogeochemical_tracers(::PISCES) (PISCES.jl:86-98)."""
import ctypes as C
import math

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
