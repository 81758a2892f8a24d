"""NonhydrostaticModel mirror: tracers under a prescribed velocity, stepped by the fused kernels.

NonhydrostaticModel(grid; biogeochemistry, advection, tracers, velocities) owns device tracer
fields (torch tensors, shape (Nz, Ny, Nx)); time_step!(model, dt) advances one Oceananigans RK3
step (three substeps, PAR recomputed from the state at every substep) through obgc_step.
Dynamics (pressure solve, closures) are outside this engine: velocities are prescribed.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from .negatives import negatives_config
from .models import replicate_of, required_biogeochemical_tracers

_PREC = {"f32": A.PREC_F32, "f64": A.PREC_F64, "mixed": A.PREC_MIXED}


class Clock:
    def __init__(self, time=0.0, iteration=0):
        self.time = time
        self.iteration = iteration


class ExplicitTimeDiscretization:
    """Oceananigans' default: the diffusive fluxes enter each RK3 stage's tendency."""


class VerticallyImplicitTimeDiscretization:
    """The vertical part is solved implicitly after each RK3 stage's explicit update."""


class ScalarDiffusivity:
    """ScalarDiffusivity([time_discretization]; κ = ...): κ a number, or f(z) sampled at the cell
    faces for the vertical part; the time discretization is ExplicitTimeDiscretization() (default)
    or VerticallyImplicitTimeDiscretization().  `horizontal` / `vertical` select
    HorizontalScalarDiffusivity / VerticalScalarDiffusivity."""

    def __init__(self, time_discretization=None, κ=0.0, ν=None, horizontal=True, vertical=True, kappa=None):
        if time_discretization is not None and not isinstance(
                time_discretization, (ExplicitTimeDiscretization, VerticallyImplicitTimeDiscretization)):
            κ, time_discretization = time_discretization, None      # ScalarDiffusivity(κ) given positionally
        self.time_discretization = time_discretization or ExplicitTimeDiscretization()
        self.kappa = κ if kappa is None else kappa
        self.horizontal, self.vertical = horizontal, vertical

    def face_values(self, grid):
        import numpy as np
        zf = -grid.Lz + grid.Lz / grid.Nz * np.arange(grid.Nz + 1)
        k = self.kappa
        return np.array([float(k(z)) for z in zf]) if callable(k) else np.full(grid.Nz + 1, float(k))


def VerticalScalarDiffusivity(time_discretization=None, κ=0.0, ν=None):
    return ScalarDiffusivity(time_discretization, κ=κ, horizontal=False)


def HorizontalScalarDiffusivity(κ=0.0, ν=None):
    return ScalarDiffusivity(κ=κ, vertical=False)


class NonhydrostaticModel:
    def __init__(self, grid, biogeochemistry, advection="WENO5", tracers=(), velocities=None,
                 precision="f32", clock=None, device="cuda", boundary_conditions=None, closure=None, forcing=None):
        """boundary_conditions: {"DIC": CarbonDioxideGasExchangeBoundaryCondition(...),
        "O2": OxygenGasExchangeBoundaryCondition(...)} as top boundary conditions (the reference's
        FieldBoundaryConditions(top = ...)); applied by time_step's fused RK3 step.  With
        CarbonateSystem(N) the keys are DIC1..DICN, each condition naming its DIC / Alk through a
        CarbonDioxideConcentration.  tracers: T and S, and any passive tracer names (at most 8
        passive tracers, CarbonateSystem replicates 2..N included).  forcing: {name: Forcing(...)}."""
        import torch
        self.grid = grid
        self.biogeochemistry = bgc = biogeochemistry
        self.precision = precision
        self.clock = clock or Clock()
        self.device = device
        self.state_dtype = torch.float32 if precision == "f32" else torch.float64
        bgc_names = list(required_biogeochemical_tracers(bgc))
        extra = [t for t in tracers if t not in bgc_names]
        # tracer codes of the C ABI: named slots; replicates 2..N of DIC / Alk and every extra tracer
        # but T and S are passive tracers (the replicates take the DIC / Alk tendency)
        self._code, source = {}, []
        for n in bgc_names:
            base = replicate_of(n)
            if base == n or n in ("DIC1", "Alk1"):
                self._code[n] = A.NAME_INDEX[base]
            else:
                self._code[n] = A.PASSIVE(len(source))
                source.append(A.NAME_INDEX[base] + 1)
        carried = [t for t in ("T", "S") if t in extra]
        for t in extra:
            if t not in carried:
                self._code[t] = A.PASSIVE(len(source))
                source.append(0)
        for t in carried:
            self._code[t] = A.NAME_INDEX[t]
        if len(source) > A.MAX_PASSIVE:
            raise ValueError(f"at most {A.MAX_PASSIVE} passive tracers (replicates included)")
        self.tracer_names = bgc_names + carried + [t for t in extra if t not in carried]
        self.tracers = {n: torch.zeros(grid.shape, dtype=self.state_dtype, device=device) for n in self.tracer_names}
        if velocities is None:
            velocities = (None, None, None)
        self.velocities = tuple(None if v is None else v.to(device=device, dtype=self.state_dtype).contiguous()
                                for v in velocities)
        self.PAR = torch.zeros(grid.shape, dtype=self.state_dtype, device=device)
        # mode (i) tendencies: one array per named tracer; a replicate shares its DIC / Alk array
        # (the functors are the same)
        self.G = {}
        for n in bgc_names:
            if self._code[n] < A.NUM_NAMED:
                self.G[n] = torch.zeros(grid.shape, dtype=self.state_dtype, device=device)
        for n in bgc_names:
            if self._code[n] >= A.NUM_NAMED:
                self.G[n] = self.G[replicate_of(n) + "1"]
        light = bgc.light_attenuation
        desc = A.ModelDesc()
        desc.npd = bgc.params
        desc.light = light.params
        desc.surface = light.surface
        desc.grid = grid.c_grid()
        desc.precision = _PREC[precision]
        desc.advection = A.ADVECTION_WENO5 if advection else A.ADVECTION_NONE
        desc.carry_T = int("T" in extra)
        desc.carry_S = int("S" in extra)
        desc.n_passive = len(source)
        for p, src in enumerate(source):
            desc.passive_tendency_of[p] = src
        desc.negatives, desc.zero_exclude, desc.invalid_fill_value = negatives_config(bgc, self.code)
        self._lib = lib = A.load()
        ctx = C.c_void_p()
        A.check(lib.obgc_create(C.byref(desc), C.byref(ctx)), "obgc_create")
        self._ctx = ctx
        self._bind()
        self.boundary_conditions = dict(boundary_conditions or {})
        for name, bc in self.boundary_conditions.items():
            name = "O2" if name == "O₂" else name
            want = A.GAS_CO2 if replicate_of(name) == "DIC" else A.GAS_O2 if name == "O2" else None
            if want is None or bc.gas != want or name not in self._code:
                raise ValueError(f"no gas exchange boundary condition of this kind for tracer {name!r}")
            wc = bc.water_concentration
            dic, alk = (self.code(wc.DIC), self.code(wc.Alk)) if want == A.GAS_CO2 else (0, 0)
            A.check(lib.obgc_set_gas_exchange_on(ctx, self._code[name], C.byref(bc.params), dic, alk),
                    "obgc_set_gas_exchange_on")
        self.forcing = dict(forcing or {})
        self._forcing_fields = {}
        for name, f in self.forcing.items():
            rate = f.field(grid, self.state_dtype, device)
            self._forcing_fields[name] = rate
            A.check(lib.obgc_set_forcing(ctx, self.code(name), C.c_void_p(rate.data_ptr()), f.start_time, f.end_time),
                    "obgc_set_forcing")
        sed = getattr(bgc, "sediment", None)
        self.sediment = sed
        if sed is not None:
            from .sediments import InstantRemineralisationSediment, SimpleMultiGSediment
            if isinstance(sed, SimpleMultiGSediment):
                names = (C.c_int32 * len(sed.sinking_nitrogen))(*[self.code(n) for n in sed.sinking_nitrogen])
                A.check(lib.obgc_set_multig_sediment(ctx, C.byref(sed.params), len(sed.sinking_nitrogen), names),
                        "obgc_set_multig_sediment")
            elif isinstance(sed, InstantRemineralisationSediment):
                names = (C.c_int32 * len(sed.sinking_tracers))(*[self.code(n) for n in sed.sinking_tracers])
                A.check(lib.obgc_set_sediment(ctx, len(sed.sinking_tracers), names,
                                              self.code(sed.remineralisation_reciever), sed.a, sed.b, sed.k),
                        "obgc_set_sediment")
            else:
                raise NotImplementedError(f"sediment model {type(sed).__name__} in the fused step")
        self.closure = closure
        if closure is not None:
            if closure.horizontal and callable(closure.kappa):
                raise ValueError("a horizontal diffusivity is a constant here")
            kh = float(closure.kappa) if closure.horizontal else 0.0
            kz = closure.face_values(grid) if closure.vertical else None
            arr = None if kz is None else (C.c_double * len(kz))(*kz)
            A.check(lib.obgc_set_diffusivity(ctx, kh, 0.0, arr), "obgc_set_diffusivity")
            if isinstance(closure.time_discretization, VerticallyImplicitTimeDiscretization):
                A.check(lib.obgc_set_vertical_time_discretization(ctx, A.VERTICALLY_IMPLICIT),
                        "obgc_set_vertical_time_discretization")

    def code(self, name):
        """The C ABI tracer code of a tracer of this model (a named slot or OBGC_PASSIVE(p))."""
        if name not in self._code:
            raise ValueError(f"name {name} not found in model.tracers.")
        return self._code[name]

    def _bind(self):
        f = A.Fields()
        for n, t in self.tracers.items():
            c = self._code[n]
            if c < A.NUM_NAMED:
                f.tracers[c] = t.data_ptr()
            else:
                f.passive[c - A.NUM_NAMED] = t.data_ptr()
        u, v, w = self.velocities
        f.u = None if u is None else u.data_ptr()
        f.v = None if v is None else v.data_ptr()
        f.w = None if w is None else w.data_ptr()
        f.PAR = self.PAR.data_ptr()
        for n, t in self.G.items():
            if self._code[n] < A.NUM_NAMED:
                f.G[self._code[n]] = t.data_ptr()
        A.check(self._lib.obgc_bind_fields(self._ctx, C.byref(f)), "obgc_bind_fields")

    def __del__(self):
        ctx = getattr(self, "_ctx", None)
        if ctx is not None and ctx.value:
            self._lib.obgc_destroy(ctx)
            self._ctx = None

    @staticmethod
    def _stream():
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    def state_array(self):
        import torch
        return torch.stack([self.tracers[n] for n in self.tracer_names])

    def set_profiling(self, on):
        A.check(self._lib.obgc_set_profiling(self._ctx, int(on)), "obgc_set_profiling")

    def sediment_fields(self, set=None):
        """SimpleMultiG: the sediment's (Ns, Nf, Nr) as FP64 numpy (3, Ny, Nx); `set` replaces them first."""
        import numpy as np
        g = self.grid
        out = np.empty((3, g.Ny, g.Nx), dtype=np.float64)
        src = None if set is None else np.ascontiguousarray(np.broadcast_to(set, (3, g.Ny, g.Nx)), dtype=np.float64)
        P = C.POINTER(C.c_double)
        A.check(self._lib.obgc_multig_sediment_state(self._ctx, None if src is None else src.ctypes.data_as(P),
                                                     out.ctypes.data_as(P)), "obgc_multig_sediment_state")
        return out

    def sediment_storage(self, set=None):
        """The sediment's storage field (Ny, Nx) as FP64 numpy; `set` replaces it first."""
        import numpy as np
        g = self.grid
        out = np.empty((g.Ny, g.Nx), dtype=np.float64)
        src = None if set is None else np.ascontiguousarray(np.broadcast_to(set, (g.Ny, g.Nx)), dtype=np.float64)
        P = C.POINTER(C.c_double)
        A.check(self._lib.obgc_sediment_storage(self._ctx, None if src is None else src.ctypes.data_as(P),
                                                out.ctypes.data_as(P)), "obgc_sediment_storage")
        return out

    def step_status(self):
        """Waits for the last step call and returns (status, OBGC_FLAG_* word) of its device-side
        checks: a NaN / infinity written into the state, an unconverged surface pCO2 solve."""
        flags = C.c_int32(0)
        rc = self._lib.obgc_step_status(self._ctx, C.byref(flags))
        return rc, flags.value

    def set_status_check(self, on):
        """Whether obgc_step waits for its kernels and returns their status (default on)."""
        A.check(self._lib.obgc_set_status_check(self._ctx, int(on)), "obgc_set_status_check")

    def set_staging(self, mode):
        """1: TMA-staged tiles when the steps qualify (default); 0: per-element cp.async staging."""
        A.check(self._lib.obgc_set_staging(self._ctx, int(mode)), "obgc_set_staging")

    def staging(self):
        """(available, last_used) of the TMA staging."""
        av, used = C.c_int32(0), C.c_int32(0)
        A.check(self._lib.obgc_get_staging(self._ctx, C.byref(av), C.byref(used)), "obgc_get_staging")
        return bool(av.value), bool(used.value)

    def set_tiling(self, levels):
        A.check(self._lib.obgc_set_tiling(self._ctx, int(levels)), "obgc_set_tiling")

    def autotune(self, dt, steps=3):
        """Time the fused step's candidate segment lengths and tile stagings on the current state
        (restored afterwards) and keep the fastest: returns (levels per item, staging, ms per step)."""
        tz, sg, ms = C.c_int32(0), C.c_int32(0), C.c_double(0)
        A.check(self._lib.obgc_autotune_step(self._ctx, self.clock.time, float(dt), int(steps), C.byref(tz), C.byref(sg),
                                             C.byref(ms), self._stream()), "obgc_autotune_step")
        return tz.value, sg.value, ms.value

    def last_timing(self):
        tot, sub, n = C.c_double(0), C.c_double(0), C.c_int64(0)
        A.check(self._lib.obgc_last_step_timing(self._ctx, C.byref(tot), C.byref(sub), C.byref(n)), "obgc_last_step_timing")
        return tot.value, sub.value, n.value

    def budget(self, group="nitrogen"):
        out = C.c_double(0)
        A.check(self._lib.obgc_tracer_budget(self._ctx, {"nitrogen": 0, "carbon": 1}[group], C.byref(out), self._stream()),
                "obgc_tracer_budget")
        return out.value


def set_(model, **values):
    """set!(model; kwargs...): numbers, numpy arrays or tensors of the grid shape."""
    import torch
    for k, v in values.items():
        if k not in model.tracers:
            raise ValueError(f"name {k} not found in model.tracers.")
        t = model.tracers[k]
        if isinstance(v, (int, float)):
            t.fill_(float(v))
        else:
            t.copy_(torch.as_tensor(v).reshape(t.shape).to(device=t.device, dtype=t.dtype))


def update_biogeochemical_state(model):
    """update_biogeochemical_state! (src/OceanBioME.jl:161-167): PAR from the current state."""
    A.check(model._lib.obgc_update_state(model._ctx, model.clock.time, model._stream()), "obgc_update_state")
    return model.PAR


def compute_tendencies(model):
    """Mode (i): the BGC tendencies of every tracer into model.G (needs a current PAR)."""
    A.check(model._lib.obgc_compute_tendencies(model._ctx, model.clock.time, model._stream()), "obgc_compute_tendencies")
    return model.G


def time_step(model, dt, nsteps=1, graph=False):
    """time_step!(model, Δt): RK3 steps through the fused kernels (a CUDA graph with graph=True)."""
    fn = model._lib.obgc_step_graph if graph else model._lib.obgc_step
    rc = fn(model._ctx, model.clock.time, float(dt), int(nsteps), model._stream())
    if rc in (A.OBGC_OK, A.ERR_NAN, A.ERR_NOT_CONVERGED):   # the steps ran: the clock moves on
        model.clock.time += dt * nsteps
        model.clock.iteration += nsteps
    A.check(rc, "obgc_step_graph" if graph else "obgc_step")
