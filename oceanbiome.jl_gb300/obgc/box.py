"""BoxModel mirror (src/BoxModel/boxmodel.jl:35-108): many independent 0-D models on the GPU."""
import ctypes as C

import numpy as np

from . import _abi as A
from .models import required_biogeochemical_tracers


class BoxModel:
    """BoxModel(; biogeochemistry, n_models, precision, forcing, prescribed_tracers).  PAR comes from the
    biogeochemistry's PrescribedPhotosyntheticallyActiveRadiation: a number, or f(t) sampled at every
    RK3 stage.  prescribed_tracers = {name: f(t) or a number}: the tracer takes f at every stage time
    and at the end of each step (update_state!, boxmodel.jl:89-106); forcing = {name: f(t) or a
    number}: a rate added to the tracer's tendency at the stage time (timesteppers.jl:59-63).  At
    most four of each; f is a function of time only (the same for every model of the batch)."""

    def __init__(self, biogeochemistry, n_models=1, precision="f64", device="cuda", params_per_model=None,
                 forcing=None, prescribed_tracers=None):
        import torch
        names = required_biogeochemical_tracers(biogeochemistry)
        self.forcing = dict(forcing or {})
        self.prescribed_tracers = dict(prescribed_tracers or {})
        for k in list(self.forcing) + list(self.prescribed_tracers):
            if k not in names:
                raise ValueError(f"name {k} not found in model.fields.")
        if len(self.forcing) > A.BOX_MAX_DRIVERS or len(self.prescribed_tracers) > A.BOX_MAX_DRIVERS:
            raise ValueError(f"at most {A.BOX_MAX_DRIVERS} forced and {A.BOX_MAX_DRIVERS} prescribed tracers")
        self.biogeochemistry = biogeochemistry
        self.n_models = n_models
        self.precision = A.PREC_F64 if precision == "f64" else A.PREC_F32
        self.state = torch.zeros((n_models, A.NUM_NAMED), dtype=torch.float64, device=device)
        self.time = 0.0
        self.iteration = 0
        self.device = device
        self.params_per_model = None
        if params_per_model is not None:
            arr = (A.NPDParams * n_models)(*params_per_model)
            buf = torch.empty(C.sizeof(arr), dtype=torch.uint8)
            C.memmove(buf.data_ptr(), C.addressof(arr), C.sizeof(arr))
            self.params_per_model = buf.to(device)

    @property
    def fields(self):
        return {n: self.state[:, A.NAME_INDEX[n]] for n in required_biogeochemical_tracers(self.biogeochemistry)}

    def set(self, **values):
        for k, v in values.items():
            if k not in required_biogeochemical_tracers(self.biogeochemistry):
                raise ValueError(f"name {k} not found in model.fields.")   # boxmodel.jl:138
            self.state[:, A.NAME_INDEX[k]] = v

    def _series(self, f, dt, nsteps, rows):
        """f(t) (or a number) at the first `rows` stage times t0 + dt (n + c_s), c = 0, 8/15, 2/3, as a
        device array [rows][n_models]."""
        import torch
        c = np.array([0.0, 8 / 15, 2 / 3])
        times = (self.time + dt * (np.arange(nsteps + 1)[:, None] + c[None, :])).ravel()[:rows]
        vals = np.full(rows, float(f)) if not callable(f) else np.array([float(f(t)) for t in times])
        return torch.as_tensor(np.repeat(vals[:, None], self.n_models, axis=1), dtype=torch.float64,
                               device=self.device).contiguous()

    def _par(self, dt, nsteps):
        import torch
        light = self.biogeochemistry.light_attenuation
        f = getattr(light, "fields", 0.0)
        if not callable(f):
            return None, float(f)
        times = self.time + dt * (np.arange(nsteps)[:, None] + np.array([0.0, 8 / 15, 2 / 3])[None, :])
        vals = np.vectorize(f)(times.ravel())
        par = np.repeat(vals[:, None], self.n_models, axis=1)
        return torch.as_tensor(par, dtype=torch.float64, device=self.device).contiguous(), 0.0

    def run(self, dt, nsteps, record_every=0, stream=0):
        """time_step!(model, dt) nsteps times; returns recorded states if record_every > 0."""
        import torch
        lib = A.load()
        par, const = self._par(dt, nsteps)
        rec = None
        if record_every > 0:
            rec = torch.zeros((nsteps // record_every, self.n_models, A.NUM_NAMED), dtype=torch.float64, device=self.device)
        ppm = None if self.params_per_model is None else self.params_per_model.data_ptr()
        d = A.BoxDrivers()
        d.PAR = None if par is None else par.data_ptr()
        d.par_constant = const
        keep = []
        for q, (k, f) in enumerate(self.prescribed_tracers.items()):
            keep.append(self._series(f, dt, nsteps, 3 * nsteps + 1))
            d.prescribed_names[q], d.prescribed[q] = A.NAME_INDEX[k], keep[-1].data_ptr()
        for q, (k, f) in enumerate(self.forcing.items()):
            keep.append(self._series(f, dt, nsteps, 3 * nsteps))
            d.forced_names[q], d.forcing[q] = A.NAME_INDEX[k], keep[-1].data_ptr()
        d.n_prescribed, d.n_forced = len(self.prescribed_tracers), len(self.forcing)
        st = C.c_void_p(stream or torch.cuda.current_stream().cuda_stream)
        A.check(lib.obgc_box_run_drivers(C.byref(self.biogeochemistry.params), ppm, self.n_models, self.state.data_ptr(),
                                         C.byref(d), self.time, float(dt), int(nsteps), int(record_every),
                                         None if rec is None else rec.data_ptr(), self.precision, st),
                "obgc_box_run_drivers")
        if keep:
            torch.cuda.synchronize()   # the series stay alive until the kernel has read them
        self.time += dt * nsteps
        self.iteration += nsteps
        return rec
