"""BoxModel mirror (src/BoxModel/boxmodel.jl:35-108): many independent 0-D models on the GPU."""
import ctypes as C

import numpy as np

from . import _abi as A
from .models import required_biogeochemical_tracers


class BoxModel:
    """BoxModel(; biogeochemistry, n_models, precision).  PAR comes from the biogeochemistry's
    PrescribedPhotosyntheticallyActiveRadiation: a number, or f(t) sampled at every RK3 stage."""

    def __init__(self, biogeochemistry, n_models=1, precision="f64", device="cuda", params_per_model=None):
        import torch
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
        A.check(lib.obgc_box_run(C.byref(self.biogeochemistry.params), ppm, self.n_models, self.state.data_ptr(),
                                 None if par is None else par.data_ptr(), const, self.time, float(dt), int(nsteps),
                                 int(record_every), None if rec is None else rec.data_ptr(), self.precision,
                                 C.c_void_p(stream or torch.cuda.current_stream().cuda_stream)), "obgc_box_run")
        self.time += dt * nsteps
        self.iteration += nsteps
        return rec
