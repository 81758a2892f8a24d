"""Many independent 1-D water columns of uneven depth, stepped together on the GPU.

Each column is the reference's single-column setup: a `RectilinearGrid(topology = (Flat, Flat,
Bounded))` with a NPZD or LOBSTER biogeochemistry, TwoBand light with a constant surface PAR,
sinking of the particulate tracers (`src/Utils/sinking_velocity_fields.jl:10-35`), a
vertically-implicit scalar diffusivity and Oceananigans' RK3 (the column examples of the
reference, e.g. `examples/column.jl`).  Columns differ in depth, level count, dt, number of steps,
maximum growth rate, surface temperature and salinity, and an optional alkalinity pulse.  LOBSTER
columns may carry the air-sea CO2 exchange of `examples/column.jl:54-64` on DIC.  The engine packs
whole columns into thread blocks and keeps each pack in shared memory for all steps of a launch.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from .negatives import negatives_config


def _stream(stream):
    if stream is not None:
        return C.c_void_p(stream)
    try:
        import torch
        if torch.cuda.is_available():
            return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    except ImportError:
        pass
    return C.c_void_p(0)


class ColumnEngine:
    """ColumnEngine(biogeochemistry; precision, max_columns, arena_cells, pack_cells, threads,
    co2_exchange).

    `arena_cells` bounds the device memory: a column of Nz levels holds Nz + 1 cells of it
    (state: n_tracers values per cell, plus one diffusivity per face).  co2_exchange: a
    CarbonDioxideGasExchangeBoundaryCondition (constant wind speed and air concentration) as the top
    condition of every column's DIC, with each column's surface temperature and salinity."""

    def __init__(self, biogeochemistry, precision="f64", max_columns=1024, arena_cells=1 << 20,
                 pack_cells=0, threads=0, light=None, co2_exchange=None):
        lib = A.load()
        d = A.ColumnsDesc()
        d.npd = biogeochemistry.params
        la = light if light is not None else biogeochemistry.light_attenuation
        d.light = la.params if la is not None else A.default_twoband()
        d.precision = {"f32": A.PREC_F32, "f64": A.PREC_F64, "mixed": A.PREC_MIXED}[precision]
        d.pack_cells = pack_cells
        d.threads = threads
        d.max_columns = max_columns
        d.arena_cells = arena_cells
        d.negatives, d.zero_exclude, d.invalid_fill_value = negatives_config(biogeochemistry)
        if co2_exchange is not None:
            d.gas_exchange = 1
            d.gas = co2_exchange.params
        self.co2_exchange = co2_exchange
        h = C.c_void_p()
        A.check(lib.obgc_columns_create(C.byref(d), C.byref(h)), "obgc_columns_create")
        self._lib, self._h = lib, h
        names = (C.c_int32 * 16)()
        n = lib.obgc_columns_tracers(h, names, 16)
        self.tracers = tuple(A.TRACER_NAMES[names[q]] for q in range(n))
        self.precision = precision
        self.slots = {}

    def close(self):
        if self._h:
            self._lib.obgc_columns_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, init, kappa, dz, dt, nsteps, surface_PAR=100.0, mu0=0.0, pulse_step=-1, pulse_k=-1,
            pulse_amount=0.0, T=15.0, S=35.0):
        """init: [n_tracers, Nz] (bottom first), or a dict name -> [Nz]; kappa: Nz + 1 face
        diffusivities (m^2/s); T, S: the surface temperature and salinity read by the CO2 exchange.
        Returns the column's slot."""
        if isinstance(init, dict):
            init = np.stack([np.asarray(init[n], dtype=np.float64) for n in self.tracers])
        init = np.ascontiguousarray(init, dtype=np.float64)
        Nz = init.shape[1]
        kappa = np.ascontiguousarray(np.broadcast_to(np.asarray(kappa, dtype=np.float64), (Nz + 1,)))
        sp = A.ColumnSpec(Nz, int(nsteps), float(dz), float(dt), float(surface_PAR), float(mu0),
                          int(pulse_step), int(pulse_k), float(pulse_amount), float(T), float(S))
        slot = C.c_int64()
        A.check(self._lib.obgc_columns_add(self._h, C.byref(sp), init.ctypes.data_as(C.POINTER(C.c_double)),
                                           kappa.ctypes.data_as(C.POINTER(C.c_double)), C.byref(slot)),
                "obgc_columns_add")
        self.slots[slot.value] = Nz
        return slot.value

    def advance(self, max_steps, stream=None):
        """Advance every unfinished column by up to max_steps steps (one kernel launch)."""
        A.check(self._lib.obgc_columns_advance(self._h, int(max_steps), _stream(stream)), "obgc_columns_advance")

    def run(self, nsteps, steps_per_launch=None, graph=True, stream=None):
        """Advance every unfinished column by up to nsteps steps in ceil(nsteps / steps_per_launch)
        launches (default: one launch), replayed from a captured CUDA graph when graph=True."""
        K = int(steps_per_launch or nsteps)
        A.check(self._lib.obgc_columns_run(self._h, int(nsteps), K, int(bool(graph)), _stream(stream)),
                "obgc_columns_run")

    def remaining(self, slot):
        left = C.c_int32()
        A.check(self._lib.obgc_columns_remaining(self._h, int(slot), C.byref(left)), "obgc_columns_remaining")
        return left.value

    def read(self, slot):
        out = np.empty((len(self.tracers), self.slots[slot]), dtype=np.float64)
        A.check(self._lib.obgc_columns_read(self._h, int(slot), out.ctypes.data_as(C.POINTER(C.c_double))),
                "obgc_columns_read")
        return out

    def remove(self, slot):
        A.check(self._lib.obgc_columns_remove(self._h, int(slot)), "obgc_columns_remove")
        self.slots.pop(slot, None)

    def autotune(self, steps=4, stream=None):
        """Time a few (threads, pack_cells) launch shapes on the resident columns (state restored)."""
        t, c = C.c_int32(), C.c_int32()
        A.check(self._lib.obgc_columns_autotune(self._h, int(steps), C.byref(t), C.byref(c), _stream(stream)),
                "obgc_columns_autotune")
        return t.value, c.value
