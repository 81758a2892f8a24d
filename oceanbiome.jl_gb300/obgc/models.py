"""NutrientsPlanktonDetritus models and the biogeochemistry plugin functions.

Mirrors src/Models/AdvectedPopulations/NutrientsPlanktonDetritus (components and constructors)
and the plugin API of src/OceanBioME.jl:100-167: required_biogeochemical_tracers,
required_biogeochemical_auxiliary_fields, biogeochemical_drift_velocity, conserved_tracers.
Parameters live in an obgc_npd_params struct (include/obgc.h) filled by the library's own presets;
the component objects only select kinds and override fields.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from .light import TwoBandPhotosyntheticallyActiveRadiation

DAY = 86400.0


class _Component:
    kind = None

    def __init__(self, **overrides):
        self.overrides = overrides


class NitrateAmmonia(_Component):
    """nutrients.jl:16-18 — NO₃ and NH₄."""
    kind = A.NUT_NITRATE_AMMONIA


class NitrateAmmoniaIron(_Component):
    """nutrients.jl:41-45 — NO₃, NH₄ and Fe."""
    kind = A.NUT_NITRATE_AMMONIA_IRON


class Nutrient(_Component):
    """nutrients.jl:81-83 — a single nutrient N."""
    kind = A.NUT_NUTRIENT


class PhytoZoo(_Component):
    """plankton.jl:19-76.  Keyword arguments override PhytoZoo fields; the formulations take
    "Linear"/"Quadratic" and light_limitation "Mondo"/"Analytical"."""


class TwoParticleAndDissolved(_Component):
    """detritus.jl:25-37,221-232 — sPOM, bPOM, DOM."""
    kind = A.DET_TWO_PARTICLE


class VariableRedfieldDetritus(_Component):
    """detritus.jl:71-81,246-257 — sPOC, bPOC, DOC, sPON, bPON, DON."""
    kind = A.DET_VARIABLE_REDFIELD


class Detritus(_Component):
    """detritus.jl:264-280 — single class D."""
    kind = A.DET_SINGLE


class CarbonateSystem(_Component):
    """carbonate_system.jl:39-83 — DIC and Alk; with N > 1 replicates the tracers DIC1..DICN and
    Alk1..AlkN, each evolving under the DIC / Alk tendency (they differ through their boundary
    conditions and forcing, e.g. an alkalinity release in one of them)."""

    def __init__(self, replicates=1):
        if int(replicates) < 1 or int(replicates) > 1 + A.MAX_PASSIVE // 2:
            raise ValueError(f"CarbonateSystem: 1 to {1 + A.MAX_PASSIVE // 2} replicates")
        self.replicates = int(replicates)
        super().__init__()


class Oxygen(_Component):
    """oxygen.jl:14-19 — O₂."""


_FORMS = {"Linear": A.LINEAR, "Quadratic": A.QUADRATIC}
_LIGHT = {"Mondo": A.LIGHT_MONDO, "MondoLightLimitation": A.LIGHT_MONDO,
          "Analytical": A.LIGHT_ANALYTICAL, "AnalyticalLightLimitation": A.LIGHT_ANALYTICAL}
# keyword names of the reference mapped to struct fields that differ in name
_ALIASES = {
    "temperature_coefficient": "temperature_coefficient",
    "redfield_ratio": "redfield_ratio",
}


def _apply(p, overrides, where):
    for k, v in overrides.items():
        if k in ("phytoplankton_mortality_formulation", "grazing_concentration_formulation"):
            setattr(p, k, _FORMS[v] if isinstance(v, str) else int(v))
        elif k == "light_limitation":
            p.light_limitation = _LIGHT[v] if isinstance(v, str) else int(v)
        elif k == "temperature_coefficient":
            if v is None:
                p.has_temperature_coefficient = 0
            else:
                p.has_temperature_coefficient = 1
                p.temperature_coefficient = float(v)
        elif k == "sinking_speed" and where == "detritus_single":
            p.detritus_sinking_speed = float(v)
        elif k == "remineralisation_rate" and where == "detritus_single":
            p.detritus_remineralisation_rate = float(v)
        elif k == "redfield_ratio" and where in ("detritus", "detritus_single"):
            p.detritus_redfield_ratio = float(v)
        elif k == "open_bottom":
            p.open_bottom = int(bool(v))
        elif hasattr(p, k):
            setattr(p, k, float(v))
        else:
            raise TypeError(f"{where}: unknown parameter {k!r}")


def preset(name):
    """The library's LOBSTER / NPZD defaults (obgc_npd_preset)."""
    lib = A.load()
    p = A.NPDParams()
    A.check(lib.obgc_npd_preset({"LOBSTER": A.PRESET_LOBSTER, "NPZD": A.PRESET_NPZD}[name], C.byref(p)), "obgc_npd_preset")
    return p


class NutrientsPlanktonDetritus:
    """The composable model (NutrientsPlanktonDetritus.jl:27-66) wrapped as the plugin's
    DiscreteBiogeochemistry (src/OceanBioME.jl:100-109)."""

    def __init__(self, grid=None, nutrients=None, plankton=None, detritus=None, carbonate_system=None,
                 oxygen=None, light_attenuation=None, sediment=None, scale_negatives=False,
                 invalid_fill_value=float("nan"), particles=None, modifiers=None, _base="LOBSTER"):
        if particles is not None:
            raise NotImplementedError("particles are outside this engine's path")
        from .sediments import InstantRemineralisationSediment, SimpleMultiGSediment
        if sediment is not None and not isinstance(sediment, (InstantRemineralisationSediment, SimpleMultiGSediment)):
            raise NotImplementedError(f"sediment model {type(sediment).__name__}: InstantRemineralisationSediment or "
                                      "SimpleMultiGSediment")
        self.sediment = sediment
        p = preset(_base)
        if nutrients is not None:
            p.nutrients = nutrients.kind
            _apply(p, nutrients.overrides, "nutrients")
        if plankton is not None:
            _apply(p, plankton.overrides, "plankton")
        if detritus is not None:
            p.detritus = detritus.kind
            _apply(p, detritus.overrides, "detritus_single" if detritus.kind == A.DET_SINGLE else "detritus")
        else:
            p.detritus = A.DET_NONE          # detritus = nothing: instant remineralisation
        p.carbonate_system = int(carbonate_system is not None)
        self.carbonate_replicates = carbonate_system.replicates if carbonate_system is not None else 0
        p.oxygen = int(oxygen is not None)
        if oxygen is not None:
            _apply(p, oxygen.overrides, "oxygen")
        self.params = p
        self.grid = grid
        if light_attenuation is None and grid is not None:
            light_attenuation = TwoBandPhotosyntheticallyActiveRadiation(grid=grid)
        self.light_attenuation = light_attenuation
        self.scale_negatives = scale_negatives
        self.invalid_fill_value = invalid_fill_value
        self.modifiers = modifiers

    # src/OceanBioME.jl:203-209
    def __repr__(self):
        names = ", ".join(":" + n for n in required_biogeochemical_tracers(self))
        kind = "NPZD" if self.params.nutrients == A.NUT_NUTRIENT else "LOBSTER"
        light = self.light_attenuation.summary() if self.light_attenuation is not None else "Nothing"
        return (f"{kind} model ({names}) \n Light attenuation: {light}\n Sediment: Nothing\n"
                f" Particles: Nothing\n Modifiers: Nothing")


def LOBSTER(grid, nutrients=None, plankton=None, detritus=None, carbonate_system=None, oxygen=None,
            surface_photosynthetically_active_radiation=None, light_attenuation=None, sediment=None,
            scale_negatives=False, invalid_fill_value=float("nan"), particles=None, modifiers=None):
    """constructors.jl:65-96."""
    if light_attenuation is None:
        light_attenuation = TwoBandPhotosyntheticallyActiveRadiation(
            grid=grid, surface_PAR=surface_photosynthetically_active_radiation)
    return NutrientsPlanktonDetritus(grid, nutrients=nutrients or NitrateAmmonia(), plankton=plankton,
                                     detritus=detritus or TwoParticleAndDissolved(),
                                     carbonate_system=carbonate_system, oxygen=oxygen,
                                     light_attenuation=light_attenuation, sediment=sediment,
                                     scale_negatives=scale_negatives, invalid_fill_value=invalid_fill_value,
                                     particles=particles, modifiers=modifiers, _base="LOBSTER")


def NPZD(grid, nutrients=None, plankton=None, detritus=None, carbonate_system=None, oxygen=None,
         surface_photosynthetically_active_radiation=None, light_attenuation=None, sediment=None,
         scale_negatives=False, invalid_fill_value=float("nan"), particles=None, modifiers=None):
    """constructors.jl:177-227 (the NPZD PhytoZoo and Detritus defaults come from the preset)."""
    if light_attenuation is None:
        light_attenuation = TwoBandPhotosyntheticallyActiveRadiation(
            grid=grid, surface_PAR=surface_photosynthetically_active_radiation)
    return NutrientsPlanktonDetritus(grid, nutrients=nutrients or Nutrient(), plankton=plankton,
                                     detritus=detritus or Detritus(), carbonate_system=carbonate_system,
                                     oxygen=oxygen, light_attenuation=light_attenuation, sediment=sediment,
                                     scale_negatives=scale_negatives, invalid_fill_value=invalid_fill_value,
                                     particles=particles, modifiers=modifiers, _base="NPZD")


# ----------------------------------------------------------------------------- plugin functions
def required_biogeochemical_tracers(bgc):
    """NutrientsPlanktonDetritus.jl:69-74 (names as in the reference, ASCII subscripts)."""
    lib = A.load()
    buf = (C.c_int32 * 32)()
    n = lib.obgc_npd_required_tracers(C.byref(bgc.params), buf, 32)
    if n < 0:
        raise A.ObgcError(-n, "obgc_npd_required_tracers")
    names = [A.ASCII_NAMES[buf[i]] for i in range(n)]
    R = getattr(bgc, "carbonate_replicates", 1)
    if R > 1:   # (DIC1, ..., DICN, Alk1, ..., AlkN) in place of (DIC, Alk) (carbonate_system.jl:47-48)
        q = names.index("DIC")
        names[q:q + 2] = [f"DIC{r}" for r in range(1, R + 1)] + [f"Alk{r}" for r in range(1, R + 1)]
    return tuple(names)


def replicate_of(name):
    """The carbonate tracer a replicate name evaluates ("DIC2" -> "DIC", "Alk1" -> "Alk"), else the
    name itself."""
    for base in ("DIC", "Alk"):
        if name.startswith(base) and name[len(base):].isdigit():
            return base
    return name


def required_biogeochemical_auxiliary_fields(bgc):
    """plankton.jl:81: PAR."""
    return ("PAR",)


def biogeochemical_drift_velocity(bgc, name, Nz=None):
    """The w-component on the Nz+1 faces (bottom first) or None (plankton.jl:60-63,
    detritus.jl:135-141,290-291)."""
    lib = A.load()
    Nz = Nz or bgc.grid.Nz
    w = np.zeros(Nz + 1)
    r = lib.obgc_npd_drift_velocity(C.byref(bgc.params), A.NAME_INDEX[replicate_of(name)], Nz,
                                    w.ctypes.data_as(C.POINTER(C.c_double)))
    if r < 0:
        raise A.ObgcError(-r, "obgc_npd_drift_velocity")
    return w if r == 1 else None


def conserved_tracers(bgc, labeled=False):
    """coupling_utils.jl:1-52: nitrogen tracers; with a carbonate system also (carbon tracers,
    scale factors)."""
    p = bgc.params
    N = ["P", "Z"] + (["N"] if p.nutrients == A.NUT_NUTRIENT else ["NO3", "NH4"])
    N += {A.DET_VARIABLE_REDFIELD: ["sPON", "bPON", "DON"], A.DET_TWO_PARTICLE: ["sPOM", "bPOM", "DOM"],
          A.DET_SINGLE: ["D"]}.get(p.detritus, [])
    if not p.carbonate_system:
        return {"nitrogen": tuple(N)} if labeled else tuple(N)
    R, rho = p.redfield_ratio, p.carbon_calcite_ratio
    Ct, Cs = ["P", "Z", "DIC"], [(1 + rho) * R, R, 1.0]
    if p.detritus == A.DET_VARIABLE_REDFIELD:
        Ct += ["sPOC", "bPOC", "DOC"]; Cs += [1.0, 1.0, 1.0]
    elif p.detritus == A.DET_TWO_PARTICLE:
        Ct += ["sPOM", "bPOM", "DOM"]; Cs += [R, R, R]
    elif p.detritus == A.DET_SINGLE:
        Ct += ["D"]; Cs += [R]
    carbon = {"tracers": tuple(Ct), "scalefactors": tuple(Cs)}
    return {"nitrogen": tuple(N), "carbon": carbon} if labeled else (tuple(N), carbon)


def eval_point(bgc, name, values, PAR, x=0.0, y=0.0, z=0.0, t=0.0):
    """Continuous-form functor (bgc)(Val(name), x, y, z, t, tracers..., PAR) at one point (host)."""
    lib = A.load()
    v = np.zeros(A.NUM_NAMED)
    for k, x_ in values.items():
        v[A.NAME_INDEX[replicate_of(k)]] = x_
    out = C.c_double(0)
    A.check(lib.obgc_npd_eval_point(C.byref(bgc.params), A.NAME_INDEX[replicate_of(name)], x, y, z, t,
                                    v.ctypes.data_as(C.POINTER(C.c_double)), PAR, C.byref(out)),
            "obgc_npd_eval_point")
    return out.value
