"""The 3-D PISCES model on the GPU against the oracle's FP64 model (or_pisces_step3d): the
update_biogeochemical_state! fields (MultiBand PAR, euphotic depth, mixed-layer PAR, calcite
saturation) and a few RK3 steps of all 26 tracers with WENO5 advection and POC/GOC sinking."""
import numpy as np
import pytest

import obgc
import oracle as O
from obgc import _abi as A
from obgc import pisces as PI
from gpuhelp import cuda, rel_err
from test_oracle_pisces import INITIAL

pytestmark = pytest.mark.gpu


def pisces_model(precision, shape=(16, 12, 10), extent=(16e3, 12e3, 400.0), seed=3, negatives=False):
    torch = cuda()
    g = obgc.RectilinearGrid(shape, extent, ("Periodic", "Periodic", "Bounded"),
                             dtype="f32" if precision == "f32" else "f64")
    bgc = PI.PISCES(g, scale_negatives=negatives)
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=seed)
    model = PI.PiscesModel(g, biogeochemistry=bgc, velocities=(u, v), precision=precision, mixed_layer_depth=-60.0)
    rng = np.random.default_rng(seed)
    zc = g.znodes()[:, None, None]
    init = {}
    for n in A.PISCES_ASCII:
        base = INITIAL[n]
        init[n] = base * np.exp(rng.normal(0, 0.2, g.shape)) if n not in ("T", "S") else np.full(g.shape, base)
    init["T"] = 4 + 10 * np.exp(zc / 80) * np.ones(g.shape)
    model.set_(**init)
    return torch, g, bgc, model, (u, v)


def tracer_errors(got, ref):
    """Per tracer max |x - x_ref| / max(|x_ref|, 1e-6 max|x_ref|), the path's error statement, for
    every tracer but CaCO3, which takes a floor of 1% of its largest value: it starts at 1e-10 and
    grows to ~1e-4 within these steps, so the cells it has not reached hold values ~1e6 below the
    rounding of the rest of the field (their absolute errors are 1e-15)."""
    return {n: rel_err(got[q], ref[q], floor_frac=1e-2 if n == "CaCO3" else 1e-6) for q, n in enumerate(A.PISCES_ASCII)}


def oracle_model(g, bgc, model, negatives=False):
    return O.pisces3d(bgc.params, g.c_grid(), model.light, model.desc.mixed_layer_depth,
                      mean_kappa=model.desc.mean_kappa, negatives=O.NEG_SCALE if negatives else O.NEG_NONE)


@pytest.mark.parametrize("precision,tol", [("mixed", 2e-5), ("f32", 2e-5)])
def test_update_state_fields_match_oracle(precision, tol):
    # light runs in FP32 arithmetic in both precisions (FP64 fields on the mixed path)
    torch, g, bgc, model, vel = pisces_model(precision)
    t = 2 * 86400.0 + 3600.0          # daytime: default_surface_PAR(t) = 100 max(0, cos(pi t / 12 h)) > 0
    model.update_state(t)
    torch.cuda.synchronize()
    s0 = model.state_array().double().cpu().numpy()
    par4, xy2, omega = O.pisces_update_state3d(oracle_model(g, bgc, model), s0, t)
    for q, name in enumerate(("PAR", "PAR1", "PAR2", "PAR3")):
        assert rel_err(model.field(name), par4[q]) < tol, name
    assert rel_err(model.field("zeu"), xy2[0]) < tol
    assert rel_err(model.field("mixed_layer_PAR"), xy2[1]) < tol
    # the carbonate solve is FP64 from the stored state in both precisions (warm-started on the
    # device); FP32 storage rounds the result
    assert rel_err(model.field("Omega"), omega) < (1e-8 if precision == "mixed" else 2e-7)
    zeu = model.field("zeu")
    assert np.all(zeu < 0) and np.any(zeu > -400.0)


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-6), ("f32", 1e-6), ("f64", 1e-10)])
def test_pisces_steps_match_oracle(precision, tol):
    # tracers relative to their own magnitude after three 20-minute RK3 steps: tendencies and light
    # are FP32 arithmetic in both precisions, so the error is the FP32 rounding of the step's changes
    torch, g, bgc, model, vel = pisces_model(precision)
    s0 = model.state_array().double().cpu().numpy()
    # daytime stages: with zero PAR and the growth rate's day length at zero (the reference evaluates
    # it with latitude and time swapped), GrowthRespirationLimitedProduction's light limitation is
    # 0/0 (growth_rate.jl:117-123) in the reference and here alike
    dt, nsteps, t0 = 1200.0, 3, 3 * 86400.0 + 3600.0
    model.time = t0
    model.time_step(dt, nsteps=nsteps)
    torch.cuda.synchronize()
    got = model.state_array().double().cpu().numpy()
    ref = np.ascontiguousarray(s0.reshape(26, -1).copy())
    u, v = (x.double().cpu().numpy().ravel().copy() for x in vel)
    O.pisces_step3d(oracle_model(g, bgc, model), ref, u=u, v=v, t=t0, dt=dt, nsteps=nsteps)
    ref = ref.reshape(got.shape)
    errs = tracer_errors(got, ref)
    # CaCO3 (floor 1% of its maximum) within 3e-6 in FP32 arithmetic
    assert errs.pop("CaCO3") < (3e-6 if precision != "f64" else tol)
    assert max(errs.values()) < tol, sorted(errs.items(), key=lambda kv: -kv[1])[:6]
    # the step changed every biogeochemical tracer, and the changes agree with the oracle's to the
    # FP32 rounding of the tendencies (T and S only move by the FP32 rounding of u_x + v_y = 0)
    moved = np.max(np.abs(ref - s0).reshape(26, -1), axis=1)
    assert np.all(moved[:24] > 0)
    change_err = np.max(np.abs((got - s0) - (ref - s0)).reshape(26, -1), axis=1) / np.maximum(moved, 1e-300)
    assert np.max(change_err[:24]) < (1e-5 if precision != "f64" else 1e-9), dict(zip(A.PISCES_ASCII, change_err))


def test_pisces_scale_negatives_match_oracle():
    # negative DOC and NH4 in some cells: ScaleNegativeTracers over the five conserved groups
    # (coupling_utils.jl:11-33) before every stage and after the step, as the oracle does.  (A
    # negative P alone would leave PChl, which no group holds, over a zero P: the chlorophyll ratio
    # PChl / (12 P + eps(0.0)) is then infinite and the reference's tendencies NaN.)
    torch, g, bgc, model, vel = pisces_model("mixed", negatives=True)
    model.tracers["DOC"][:, :2, :3] = -0.05
    model.tracers["NH4"][:, 3:5, 4:6] = -0.01
    s0 = model.state_array().double().cpu().numpy()
    model.time_step(600.0, nsteps=1)
    torch.cuda.synchronize()
    got = model.state_array().double().cpu().numpy()
    ref = np.ascontiguousarray(s0.reshape(26, -1).copy())
    u, v = (x.double().cpu().numpy().ravel().copy() for x in vel)
    O.pisces_step3d(oracle_model(g, bgc, model, negatives=True), ref, u=u, v=v, t=0.0, dt=600.0, nsteps=1)
    ref = ref.reshape(got.shape)
    assert np.all(np.isfinite(got))
    for name in ("DOC", "NH4"):
        assert got[A.PISCES_INDEX[name]].min() >= 0, name
    errs = tracer_errors(got, ref)
    assert errs.pop("CaCO3") < 1e-5      # 3.4e-6: FP32 light and tendencies on a 1e-10 start
    # the two tracers made negative: ScaleNegativeTracers leaves cells near zero where the FP32
    # tendencies' rounding is large against the value (3.8e-6 for DOC)
    assert max(errs.pop("DOC"), errs.pop("NH4")) < 1e-5
    assert max(errs.values()) < 1e-6, sorted(errs.items(), key=lambda kv: -kv[1])[:6]


@pytest.mark.parametrize("precision", ["f64", "mixed", "f32"])
def test_pisces_many_steps_on_a_config4_subdomain(precision):
    """100 steps of 20 minutes on a 32 x 32 x 48 piece of the 128 x 128 x 48 configuration (same
    dx, dy, dz; 3-band MultiBand light at a constant surface PAR of 100 W/m2, random-streamfunction
    velocity, depth-profile initial conditions with 5% noise) against the oracle's FP64 model."""
    torch = cuda()
    shape, extent, steps = (32, 32, 48), (25_000.0, 25_000.0, 1000.0), 100
    g = obgc.RectilinearGrid(shape, extent, ("Periodic", "Periodic", "Bounded"), dtype="f32" if precision == "f32" else "f64")
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=4)
    pm = obgc.PiscesModel(g, biogeochemistry=obgc.PISCES(g), velocities=(u, v), precision=precision,
                          mixed_layer_depth=-50.0, surface_PAR=100.0)
    pm.set_(**obgc.pisces_initial_conditions(g, seed=5))
    s0 = pm.state_array().double().cpu().numpy()
    pm.time_step(1200.0, nsteps=steps)
    torch.cuda.synchronize()
    got = pm.state_array().double().cpu().numpy()
    assert np.all(np.isfinite(got))
    om = O.pisces3d(pm.bgc.params, g.c_grid(), pm.light, -50.0, surface_kind=A.SURFACE_CONSTANT, surface_value=100.0)
    ref = np.ascontiguousarray(s0.reshape(26, -1).copy())
    O.pisces_step3d(om, ref, u=u.double().cpu().numpy().ravel().copy(), v=v.double().cpu().numpy().ravel().copy(),
                    t=0.0, dt=1200.0, nsteps=steps)
    ref = ref.reshape(got.shape)
    norm = {n: float(np.linalg.norm(got[q] - ref[q]) / np.linalg.norm(ref[q])) for q, n in enumerate(A.PISCES_ASCII)}
    cell = tracer_errors(got, ref)
    print(precision, "worst cellwise", max(cell.items(), key=lambda kv: kv[1]), "normwise", max(norm.items(), key=lambda kv: kv[1]))
    tol_norm, tol_cell = {"f64": (1e-9, 1e-7), "mixed": (1e-5, 1e-3), "f32": (1e-5, 1e-3)}[precision]
    assert max(norm.values()) < tol_norm, sorted(norm.items(), key=lambda kv: -kv[1])[:5]
    assert max(cell.values()) < tol_cell, sorted(cell.items(), key=lambda kv: -kv[1])[:5]
