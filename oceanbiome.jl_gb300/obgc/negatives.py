"""Negative-tracer modifiers (src/Utils/negative_tracers.jl).

`ScaleNegativeTracers` rescales a conserved group so that no member is negative while the group's
scaled total is kept; `ZeroNegativeTracers` clips every tracer not excluded at zero.  A model built
with `scale_negatives=True` (constructors.jl:20, NutrientsPlanktonDetritus.jl:50-59) or with one of
these as `modifiers` applies it on the device to the initial state and after every RK3 stage, as
Oceananigans' update_state! does.  Each modifier can also be applied once to a set of fields.
"""
import ctypes as C
import math

from . import _abi as A


class ScaleNegativeTracers:
    """ScaleNegativeTracers(tracers; scalefactors = ones, invalid_fill_value = NaN, warn = false)
    (negative_tracers.jl:75-81)."""

    def __init__(self, tracers, scalefactors=None, invalid_fill_value=math.nan, warn=False):
        if warn:
            raise NotImplementedError("Warning not currently implemented")          # negative_tracers.jl:55
        tracers = tuple(tracers)
        scalefactors = tuple(scalefactors) if scalefactors is not None else (1.0,) * len(tracers)
        if len(scalefactors) != len(tracers):
            raise ValueError("Incorrect number of scale factors provided")          # negative_tracers.jl:77
        self.tracers, self.scalefactors, self.invalid_fill_value = tracers, scalefactors, invalid_fill_value

    def summary(self):
        return f"Mass conserving negative scaling of {self.tracers}"

    def apply(self, fields, grid, stream=0):
        """Apply once to `fields` (name -> device tensor on `grid`)."""
        ptrs = (C.c_void_p * len(self.tracers))(*[fields[n].data_ptr() for n in self.tracers])
        sf = (C.c_double * len(self.tracers))(*self.scalefactors)
        dtype = A.F32 if str(fields[self.tracers[0]].dtype).endswith("float32") else A.F64
        A.check(A.load().obgc_scale_negatives(C.byref(grid.c_grid()), dtype, len(self.tracers), ptrs, sf,
                                              self.invalid_fill_value, C.c_void_p(stream)), "obgc_scale_negatives")


class ZeroNegativeTracers:
    """ZeroNegativeTracers(; exclude = ()) (negative_tracers.jl:13-21)."""

    def __init__(self, exclude=()):
        self.exclude = tuple(exclude)

    def summary(self):
        return "ZeroNegativeTracers"

    def apply(self, fields, grid, stream=0):
        names = [n for n in fields if n not in self.exclude]
        ptrs = (C.c_void_p * len(names))(*[fields[n].data_ptr() for n in names])
        dtype = A.F32 if str(fields[names[0]].dtype).endswith("float32") else A.F64
        A.check(A.load().obgc_zero_negatives(C.byref(grid.c_grid()), dtype, len(names), ptrs, C.c_void_p(stream)),
                "obgc_zero_negatives")


def negatives_config(bgc, code=None):
    """(mode, zero_exclude mask, invalid_fill_value) of a biogeochemistry's modifier for the engine:
    scale_negatives = true scales conserved_tracers(bgc); a ZeroNegativeTracers modifier zeroes.
    code: a model's tracer-name -> C ABI code map (passive tracers have bits 21 + p)."""
    if getattr(bgc, "scale_negatives", False):
        return A.NEGATIVES_SCALE, 0, float(getattr(bgc, "invalid_fill_value", math.nan))
    mods = getattr(bgc, "modifiers", None)
    mods = mods if isinstance(mods, tuple) else (mods,)
    for m in mods:
        if isinstance(m, ZeroNegativeTracers):
            mask = 0
            for n in m.exclude:
                mask |= 1 << (code(n) if code is not None else A.NAME_INDEX[n])
            return A.NEGATIVES_ZERO, mask, math.nan
        if isinstance(m, ScaleNegativeTracers):
            raise NotImplementedError("a custom ScaleNegativeTracers group as a model modifier: use scale_negatives=True "
                                      "(conserved_tracers) or apply() it between steps")
    return A.NEGATIVES_NONE, 0, math.nan
