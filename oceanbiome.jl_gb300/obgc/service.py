"""Continuous-batching service for column runs (the C ABI's obgc_service_*).

Requests are submitted from any thread and return at once; a native worker thread admits them into
the packed column engine while a slot and arena space (the HBM budget) are free, advances every
resident run by `chunk_steps` steps per launch with two launches queued, and hands each finished
run back with its latency (submit to result).  A run's result does not depend on the runs it
shares launches with: it equals the same run stepped alone in a ColumnEngine of the same precision.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from .negatives import negatives_config


class ColumnService:
    def __init__(self, biogeochemistry, precision="f32", max_columns=4096, arena_cells=1 << 20, chunk_steps=32,
                 max_queue=0, pack_cells=0, threads=0, light=None, co2_exchange=None):
        """co2_exchange: a CarbonDioxideGasExchangeBoundaryCondition on every LOBSTER run's DIC (the
        uptake an alkalinity release drives), with each request's surface T and S."""
        lib = A.load()
        d = A.ServiceDesc()
        c = d.columns
        c.npd = biogeochemistry.params
        la = light if light is not None else biogeochemistry.light_attenuation
        c.light = la.params if la is not None else A.default_twoband()
        c.precision = {"f32": A.PREC_F32, "f64": A.PREC_F64, "mixed": A.PREC_MIXED}[precision]
        c.pack_cells = pack_cells
        c.threads = threads
        c.max_columns = max_columns
        c.arena_cells = arena_cells
        c.negatives, c.zero_exclude, c.invalid_fill_value = negatives_config(biogeochemistry)
        if co2_exchange is not None:
            c.gas_exchange = 1
            c.gas = co2_exchange.params
        self.co2_exchange = co2_exchange
        d.chunk_steps = chunk_steps
        d.max_queue = max_queue
        h = C.c_void_p()
        A.check(lib.obgc_service_create(C.byref(d), C.byref(h)), "obgc_service_create")
        self._lib, self._h = lib, h
        eng = C.c_void_p()
        A.check(lib.obgc_service_engine(h, C.byref(eng)), "obgc_service_engine")
        names = (C.c_int32 * 16)()
        n = lib.obgc_columns_tracers(eng, names, 16)
        self.tracers = tuple(A.TRACER_NAMES[names[q]] for q in range(n))
        self._levels = {}

    def close(self):
        if self._h:
            self._lib.obgc_service_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, init, kappa, dz, dt, nsteps, surface_PAR=100.0, mu0=0.0, pulse_step=-1, pulse_k=-1,
               pulse_amount=0.0, T=15.0, S=35.0):
        if isinstance(init, dict):
            init = np.stack([np.asarray(init[n], dtype=np.float64) for n in self.tracers])
        init = np.ascontiguousarray(init, dtype=np.float64)
        Nz = init.shape[1]
        kappa = np.ascontiguousarray(np.broadcast_to(np.asarray(kappa, dtype=np.float64), (Nz + 1,)))
        sp = A.ColumnSpec(Nz, int(nsteps), float(dz), float(dt), float(surface_PAR), float(mu0), int(pulse_step),
                          int(pulse_k), float(pulse_amount), float(T), float(S))
        rid = C.c_int64()
        A.check(self._lib.obgc_service_submit(self._h, C.byref(sp), init.ctypes.data_as(C.POINTER(C.c_double)),
                                              kappa.ctypes.data_as(C.POINTER(C.c_double)), C.byref(rid)),
                "obgc_service_submit")
        self._levels[rid.value] = Nz
        return rid.value

    def submit_request(self, r):
        """Submit a dict as made by lobster_column_request / npzd_column_ensemble."""
        return self.submit(r["init"], r["kappa"], r["dz"], r["dt"], r["nsteps"], surface_PAR=r["surface_PAR"],
                           mu0=r.get("mu0", 0.0), pulse_step=r.get("pulse_step", -1), pulse_k=r.get("pulse_k", -1),
                           pulse_amount=r.get("pulse_amount", 0.0), T=r.get("T", 15.0), S=r.get("S", 35.0))

    def wait(self, rid, timeout=600.0):
        """(final state [n_tracers, Nz], latency in ms)."""
        Nz = self._levels.get(rid)
        out = np.empty((len(self.tracers), Nz), dtype=np.float64) if Nz is not None else None
        ptr = out.ctypes.data_as(C.POINTER(C.c_double)) if out is not None else None
        lat = C.c_double()
        A.check(self._lib.obgc_service_wait(self._h, int(rid), float(timeout), ptr, C.byref(lat)), "obgc_service_wait")
        self._levels.pop(rid, None)
        return out, lat.value

    def drain(self, timeout=600.0):
        A.check(self._lib.obgc_service_drain(self._h, float(timeout)), "obgc_service_drain")

    def stats(self):
        s = A.ServiceStats()
        A.check(self._lib.obgc_service_get_stats(self._h, C.byref(s)), "obgc_service_get_stats")
        return {f: getattr(s, f) for f, _ in s._fields_}

    def reset_stats(self):
        A.check(self._lib.obgc_service_reset_stats(self._h), "obgc_service_reset_stats")
