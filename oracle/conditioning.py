"""TEST INFRASTRUCTURE (the oracle): the long-run error statement of the 3-D LOBSTER + carbonates
path and the oracle's own conditioning envelope.

The 3-D step of the reference (WENO5 advection, src/OceanBioME.jl:157-159 inside Oceananigans'
tracer tendency, with the NutrientsPlanktonDetritus functors and TwoBand light) is evaluated here
by the FP64 oracle (or_step.c).  Over 1000 steps its answer is sensitive to rounding: the WENO5-Z
smoothness weights of a rough field react to changes of one unit in the last place, and a
perturbation of that size grows into cell differences of 1e-5 and more (the BGC functors alone
keep it at 1e-15).  The envelope runs put that on record: the oracle itself, with every stored
value multiplied by (1 +/- r) after every RK3 stage (or_model3d.stage_rounding, a seeded sign per
value and stage), for r one FP64 unit roundoff (2^-53) and one FP32 unit roundoff (2^-24).  Any
implementation that rounds differently from the oracle differs from it by about the first; any
that rounds to FP32 anywhere in the update by about the second.

Only tests/ and bench.py's accuracy legs use this module, as the oracle.
"""
import os
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_HERE)
for _p in (_HERE, _ROOT, os.path.join(_ROOT, "oceanbiome.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import oracle as O          # noqa: E402
from obgc import _abi as A  # noqa: E402

NAMES = ["NO3", "NH4", "P", "Z", "sPOM", "bPOM", "DOM", "DIC", "Alk", "T", "S"]
FULL_SHAPE = (256, 256, 64)
FULL_EXTENT = (50_000.0, 50_000.0, 500.0)
DT = 300.0
U32 = 2.0 ** -24   # FP32 unit roundoff
U64 = 2.0 ** -53   # FP64 unit roundoff


def error_statement(got, ref, names=NAMES):
    """Per tracer: max |x - x_ref|; the cellwise max |x - x_ref| / max(|x_ref|, 1e-6 max|x_ref|);
    and the normwise ||x - x_ref||_2 / ||x_ref||_2."""
    out = {}
    for q, n in enumerate(names):
        g, r = np.asarray(got[q], dtype=np.float64), np.asarray(ref[q], dtype=np.float64)
        d = np.abs(g - r)
        floor = 1e-6 * max(float(np.max(np.abs(r))), 1e-300)
        out[n] = {"max_abs": float(d.max()), "max_rel": float(np.max(d / np.maximum(np.abs(r), floor))),
                  "norm_rel": float(np.linalg.norm((g - r).ravel()) / max(np.linalg.norm(r.ravel()), 1e-300))}
    return out


def ph_total(state, names=NAMES, threads=None):
    """FP64 pH (total scale) of every cell from the state's DIC, Alk, T and S (the oracle's
    CarbonChemistry, carbon_chemistry.jl:4-218)."""
    o = O.carbon_options(output=A.OUT_PH_TOTAL)
    f = {n: np.ascontiguousarray(np.asarray(state[names.index(n)], dtype=np.float64).ravel()) for n in ("DIC", "Alk", "T", "S")}
    return O.carbon_chemistry_batch(o, f["DIC"], f["Alk"], f["T"], f["S"], threads=threads)


def summary(stmt, ph=None, ph_ref=None):
    """Worst tracer of each measure, and the pH differences (max and RMS)."""
    s = {k: max(v[k] for v in stmt.values()) for k in ("max_rel", "norm_rel")}
    s["max_rel_tracer"] = max(stmt, key=lambda n: stmt[n]["max_rel"])
    s["norm_rel_tracer"] = max(stmt, key=lambda n: stmt[n]["norm_rel"])
    if ph is not None:
        d = np.asarray(ph) - np.asarray(ph_ref)
        s["pH_max_abs"] = float(np.max(np.abs(d)))
        s["pH_rms"] = float(np.sqrt(np.mean(d * d)))
    return s


class LobsterCase:
    """The headline workload's physics on a smaller grid: LOBSTER + carbonates, T and S, extent
    scaled with the grid so that dx and dy are those of the 256 x 256 x 64 configuration,
    random-streamfunction velocity (0.1 m/s RMS), seeded initial conditions, TwoBand light with the
    default surface PAR, dt = 300 s."""

    def __init__(self, shape=(32, 32, 16), vel_seed=3, init_seed=4):
        import obgc
        self.shape = tuple(shape)
        ext = (FULL_EXTENT[0] * shape[0] / FULL_SHAPE[0], FULL_EXTENT[1] * shape[1] / FULL_SHAPE[1], FULL_EXTENT[2])
        self.extent = ext
        self.grid = obgc.RectilinearGrid(shape, ext, ("Periodic", "Periodic", "Bounded"), dtype="f64")
        self.bgc = obgc.LOBSTER(self.grid, carbonate_system=obgc.CarbonateSystem())
        u, v, _ = obgc.random_streamfunction_velocity(self.grid, rms=0.1, seed=vel_seed, device="cpu")
        self.u = np.ascontiguousarray(u.numpy().ravel())
        self.v = np.ascontiguousarray(v.numpy().ravel())
        self.vel_seed = vel_seed
        self.init = obgc.lobster_initial_conditions(self.grid, seed=init_seed)
        self.state0 = np.ascontiguousarray(np.stack(
            [np.broadcast_to(np.asarray(self.init[n], dtype=np.float64), self.grid.shape) for n in NAMES]))

    def oracle_run(self, steps, stage_rounding=0.0, seed=0, threads=None):
        m = O.model3d(self.bgc.params, self.grid.c_grid(), NAMES)
        m.stage_rounding = stage_rounding
        m.rounding_seed = seed
        s = self.state0.copy()
        O.step3d(m, s, u=self.u, v=self.v, t=0.0, dt=DT, nsteps=steps, threads=threads)
        return s

    def envelope(self, ref, ph_ref, steps, rounding, seeds, threads=None):
        """The largest difference from `ref` over oracle runs with per-stage rounding `rounding`
        under each seed: worst cellwise and normwise relative error over tracers, pH max and RMS."""
        env = {"max_rel": 0.0, "norm_rel": 0.0, "pH_max_abs": 0.0, "pH_rms": 0.0}
        for sd in seeds:
            s = self.oracle_run(steps, stage_rounding=rounding, seed=sd, threads=threads)
            sm = summary(error_statement(s, ref), ph_total(s, threads=threads), ph_ref)
            for k in env:
                env[k] = max(env[k], sm[k])
        env["rounding"] = rounding
        env["seeds"] = list(seeds)
        return env
