"""Light attenuation models (src/Light): TwoBand, MultiBand and Prescribed PAR."""
import ctypes as C

import numpy as np

from . import _abi as A

# Morel (1988) coefficients at 5 nm from 350 to 700 nm (the table of src/Light/
# morel_coefficients.jl / multi_band.jl:209-239), used for the default MultiBand band means.
MOREL_LAMBDA = np.arange(350, 701, 5, dtype=np.float64)
MOREL_KW = np.array([
    0.0271, 0.0238, 0.0216, 0.0188, 0.0177, 0.01595, 0.0151, 0.01376, 0.01271, 0.01208,
    0.01042, 0.0089, 0.00812, 0.00765, 0.00758, 0.00768, 0.0077, 0.00792, 0.00885, 0.0099,
    0.01148, 0.01182, 0.01188, 0.01211, 0.01251, 0.0132, 0.01444, 0.01526, 0.0166, 0.01885,
    0.02188, 0.02701, 0.03385, 0.0409, 0.04214, 0.04287, 0.04454, 0.0463, 0.04846, 0.05212,
    0.05746, 0.06053, 0.0628, 0.06507, 0.07034, 0.07801, 0.09038, 0.11076, 0.13584, 0.16792,
    0.2231, 0.25838, 0.26506, 0.26843, 0.27612, 0.284, 0.29218, 0.30176, 0.31134, 0.32553,
    0.34052, 0.3715, 0.41048, 0.42947, 0.43946, 0.44844, 0.46543, 0.48642, 0.5164, 0.55939, 0.62438])
MOREL_E = np.array([
    0.778, 0.767, 0.756, 0.737, 0.72, 0.7, 0.685, 0.673, 0.67, 0.66,
    0.64358, 0.64776, 0.65175, 0.65555, 0.65917, 0.66259, 0.66583, 0.66889, 0.67175, 0.67443,
    0.67692, 0.67923, 0.68134, 0.68327, 0.68501, 0.68657, 0.68794, 0.68903, 0.68955, 0.68947,
    0.6888, 0.68753, 0.68567, 0.6832, 0.68015, 0.67649, 0.67224, 0.66739, 0.66195, 0.65591,
    0.64927, 0.64204, 0.64, 0.63, 0.623, 0.615, 0.61, 0.614, 0.618, 0.622,
    0.626, 0.63, 0.634, 0.638, 0.642, 0.647, 0.653, 0.658, 0.663, 0.667,
    0.672, 0.677, 0.682, 0.687, 0.695, 0.697, 0.693, 0.665, 0.64, 0.62, 0.6])
MOREL_CHI = np.array([
    0.153, 0.149, 0.144, 0.14, 0.136, 0.131, 0.127, 0.123, 0.119, 0.118,
    0.11748, 0.12066, 0.12259, 0.12326, 0.12269, 0.12086, 0.11779, 0.11372, 0.10963, 0.1056,
    0.10165, 0.09776, 0.09393, 0.09018, 0.08649, 0.08287, 0.07932, 0.07584, 0.07242, 0.06907,
    0.06579, 0.06257, 0.05943, 0.05635, 0.05341, 0.05072, 0.04829, 0.04611, 0.04419, 0.04253,
    0.04111, 0.03996, 0.039, 0.0375, 0.036, 0.034, 0.033, 0.0328, 0.0325, 0.033,
    0.034, 0.035, 0.036, 0.0375, 0.0385, 0.04, 0.042, 0.043, 0.044, 0.0445,
    0.045, 0.046, 0.0475, 0.049, 0.0515, 0.052, 0.0505, 0.044, 0.039, 0.034, 0.03])


def default_surface_PAR(t):
    """Light.jl:45-47."""
    return 100 * max(0.0, np.cos(t * np.pi / (12 * 3600.0)))


def _surface(surface_PAR):
    s = A.Surface()
    if surface_PAR is None or surface_PAR is default_surface_PAR:
        s.kind = A.SURFACE_DEFAULT
    elif isinstance(surface_PAR, (int, float)):
        s.kind, s.value = A.SURFACE_CONSTANT, float(surface_PAR)
    else:   # a per-column device tensor (discrete / field form)
        s.kind, s.field = A.SURFACE_FIELD, surface_PAR.data_ptr()
    return s


class TwoBandPhotosyntheticallyActiveRadiation:
    """2band.jl:106-146.  surface_PAR: None (default_surface_PAR), a number, or a per-column
    tensor (Nx*Ny) of the grid's dtype."""

    def __init__(self, grid=None, water_red_attenuation=0.225, water_blue_attenuation=0.0232,
                 chlorophyll_red_attenuation=0.037, chlorophyll_blue_attenuation=0.074,
                 chlorophyll_red_exponent=0.629, chlorophyll_blue_exponent=0.674, pigment_ratio=0.7,
                 phytoplankton_chlorophyll_ratio=1.31, surface_PAR=None):
        self.grid = grid
        self.params = A.TwoBandParams(water_red_attenuation, water_blue_attenuation,
                                      chlorophyll_red_attenuation, chlorophyll_blue_attenuation,
                                      chlorophyll_red_exponent, chlorophyll_blue_exponent, pigment_ratio,
                                      phytoplankton_chlorophyll_ratio)
        self.surface_PAR = surface_PAR
        self.surface = _surface(surface_PAR)
        self.field = None

    def summary(self):
        return f"Two-band light attenuation model ({'Float32' if self.grid is not None and self.grid.dtype == 'f32' else 'Float64'})"

    def compute(self, P, PAR, t=0.0, stream=0):
        """update_TwoBandPhotosyntheticallyActiveRadiation! into PAR (device tensors)."""
        import torch
        lib = A.load()
        g = self.grid.c_grid()
        dt = A.F32 if P.dtype == torch.float32 else A.F64
        A.check(lib.obgc_twoband_par(C.byref(self.params), C.byref(self.surface), C.byref(g), dt, P.data_ptr(),
                                     PAR.data_ptr(), float(t), C.c_void_p(stream)), "obgc_twoband_par")
        return PAR


def numerical_mean_coefficients(bands, base_bands=MOREL_LAMBDA, kw=MOREL_KW, e=MOREL_E, chi=MOREL_CHI):
    """Band means of multi_band.jl:93-104,136-140 through the library."""
    lib = A.load()
    n = len(bands)
    edges = np.array([x for b in bands for x in b], dtype=np.float64)
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (base_bands, kw, e, chi)]
    okw, oe, ochi = np.zeros(n), np.zeros(n), np.zeros(n)
    P = C.POINTER(C.c_double)
    A.check(lib.obgc_multiband_coefficients(n, edges.ctypes.data_as(P), len(arrs[0]), *[a.ctypes.data_as(P) for a in arrs],
                                            okw.ctypes.data_as(P), oe.ctypes.data_as(P), ochi.ctypes.data_as(P)),
            "obgc_multiband_coefficients")
    return okw, oe, ochi


class MultiBandPhotosyntheticallyActiveRadiation:
    """multi_band.jl:80-134: bands in nm, coefficients averaged from the base tables."""

    def __init__(self, grid=None, bands=((400, 500), (500, 600), (600, 700)), base_bands=MOREL_LAMBDA,
                 base_water_attenuation_coefficient=MOREL_KW, base_chlorophyll_exponent=MOREL_E,
                 base_chlorophyll_attenuation_coefficient=MOREL_CHI, surface_PAR=None,
                 surface_PAR_division=None):
        self.grid = grid
        self.bands = tuple(bands)
        n = len(self.bands)
        self.kw, self.e, self.chi = numerical_mean_coefficients(
            self.bands, base_bands, base_water_attenuation_coefficient, base_chlorophyll_exponent,
            base_chlorophyll_attenuation_coefficient)
        self.division = np.full(n, 1.0 / n) if surface_PAR_division is None else np.asarray(surface_PAR_division, dtype=np.float64)
        if self.division.sum() != 1:
            raise ValueError("surface_PAR_division does not sum to 1")   # multi_band.jl:106
        self.surface_PAR = surface_PAR
        self.surface = _surface(surface_PAR)

    def summary(self):
        names = tuple(f"PAR{n + 1}" for n in range(len(self.bands)))
        return f"Multi band light attenuation model with {len(self.bands)} bands {names}"

    def compute(self, Chl, band_fields, total=None, t=0.0, stream=0):
        import torch
        lib = A.load()
        g = self.grid.c_grid()
        n = len(self.bands)
        P = C.POINTER(C.c_double)
        ptrs = (C.c_void_p * n)(*[f.data_ptr() for f in band_fields])
        dt = A.F32 if Chl.dtype == torch.float32 else A.F64
        A.check(lib.obgc_multiband_par(n, self.kw.ctypes.data_as(P), self.e.ctypes.data_as(P), self.chi.ctypes.data_as(P),
                                       self.division.ctypes.data_as(P), C.byref(self.surface), C.byref(g), dt,
                                       Chl.data_ptr(), ptrs, None if total is None else total.data_ptr(), float(t),
                                       C.c_void_p(stream)), "obgc_multiband_par")
        return band_fields, total


class PrescribedPhotosyntheticallyActiveRadiation:
    """prescribed.jl:25-46: PAR supplied by the caller (a tensor, a number, or f(t))."""

    def __init__(self, fields):
        self.fields = fields

    def summary(self):
        return "Prescribed PAR"

    def value(self, t):
        return self.fields(t) if callable(self.fields) else self.fields


def euphotic_depth(grid, PAR, zeu, surface_PAR=None, cutoff=1e-3, t=0.0, stream=0):
    """compute_euphotic_depth! (compute_euphotic_depth.jl:3-39) into zeu (Nx*Ny)."""
    import torch
    lib = A.load()
    s = _surface(surface_PAR)
    g = grid.c_grid()
    dt = A.F32 if PAR.dtype == torch.float32 else A.F64
    A.check(lib.obgc_euphotic_depth(C.byref(s), C.byref(g), dt, PAR.data_ptr(), zeu.data_ptr(), cutoff, float(t),
                                    C.c_void_p(stream)), "obgc_euphotic_depth")
    return zeu
