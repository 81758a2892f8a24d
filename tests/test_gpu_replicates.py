"""CarbonateSystem(N) replicates, passive tracers and tracer forcing in the fused 3-D step, on the
GPU against the oracle.

The reference's own case (test/test_gasexchange_carbon_chem.jl:38-67, examples/oae_experiment.jl):
LOBSTER with CarbonateSystem(2), a CO2 gas-exchange condition on DIC1 (water CO2 from DIC1/Alk1)
and one on DIC2 (from DIC2/Alk2), and an alkalinity release forcing Alk2 inside a region over a
window of time.  The replicates DIC2 / Alk2 run as passive tracers taking the DIC / Alk tendency of
the same stage; a further passive tracer C has no BGC tendency."""
import ctypes as C
import math

import numpy as np
import pytest

import obgc
import oracle as O
from obgc import _abi as A
from gpuhelp import cuda, rel_err

pytestmark = pytest.mark.gpu
# C starts as noise of both signs: its error is measured against 1 % of its largest magnitude where
# it crosses zero (the other tracers keep one sign)
FLOOR = {"C": 1e-2}


def oracle_layout(model):
    """Oracle names (None for passive slots) and tendency sources of a model's tracer order."""
    names, src = [], {}
    for q, n in enumerate(model.tracer_names):
        c = model.code(n)
        if c < A.NUM_NAMED:
            names.append(A.TRACER_NAMES[c])
        else:
            names.append(None)
            base = obgc.models.replicate_of(n)
            if base != n:
                src[q] = base
    return names, src


def oae_model(precision, shape=(24, 16, 8), seed=5, with_bcs=True, with_forcing=True, modifiers=None):
    torch = cuda()
    # 208 m cells: the flow (0.27 m/s at most) moves under 0.4 cells per 300 s step
    g = obgc.RectilinearGrid(shape, (5000.0, 4000.0, 15.0), dtype="f32" if precision == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(2), modifiers=modifiers)
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=seed)
    bcs = {}
    if with_bcs:
        for r in (1, 2):
            wc = obgc.CarbonDioxideConcentration(DIC=f"DIC{r}", Alk=f"Alk{r}")
            bcs[f"DIC{r}"] = obgc.CarbonDioxideGasExchangeBoundaryCondition(wind_speed=5.0, water_concentration=wc)
    forcing = {}
    if with_forcing:
        z, y, x = g.nodes()
        mask = ((x[None, None, :] - 2500) ** 2 + (y[None, :, None] - 2000) ** 2 < 1000.0 ** 2) & (z[:, None, None] > -4)
        rate = np.where(mask, 0.05, 0.0) * np.ones(g.shape)
        forcing["Alk2"] = obgc.Forcing(rate, start_time=400.0, end_time=1000.0)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S", "C"), velocities=(u, v, None),
                                     precision=precision, boundary_conditions=bcs, forcing=forcing)
    init = obgc.lobster_initial_conditions(g, seed=seed + 1)
    rng = np.random.default_rng(seed)
    vals = {k: val for k, val in init.items() if k in model.tracers}
    vals.update(DIC1=init["DIC"], Alk1=init["Alk"], DIC2=np.asarray(init["DIC"]) + 1.0,
                Alk2=np.asarray(init["Alk"]) + 1.0, C=rng.uniform(-1, 1, g.shape))
    obgc.set_(model, **vals)
    return g, bgc, model, (u, v), bcs, forcing


def oracle_run(model, bgc, g, vel, s0, dt, nsteps, bcs=None, forcing=None):
    names, src = oracle_layout(model)
    slot = {n: q for q, n in enumerate(model.tracer_names)}
    gas = [(bc.params, slot[name], slot[bc.water_concentration.DIC], slot[bc.water_concentration.Alk])
           for name, bc in (bcs or {}).items()]
    frc = {slot[n]: (np.asarray(f.rate, dtype=np.float64), f.start_time, f.end_time) for n, f in (forcing or {}).items()}
    m = O.model3d(bgc.params, g.c_grid(), names, gas_exchange=gas, tendency_of=src, forcing=frc)
    ref = np.ascontiguousarray(s0.copy())
    u, v = (x.double().cpu().numpy().ravel().copy() for x in vel)
    O.step3d(m, ref, u=u, v=v, t=0.0, dt=dt, nsteps=nsteps)
    return ref


def test_tracer_order_and_codes():
    cuda()
    g = obgc.RectilinearGrid((8, 8, 4), (1000.0, 1000.0, 10.0))
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(2))
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S", "C"))
    assert model.tracer_names[7:] == ["DIC1", "DIC2", "Alk1", "Alk2", "T", "S", "C"]
    assert model.code("DIC1") == A.NAME_INDEX["DIC"] and model.code("Alk1") == A.NAME_INDEX["Alk"]
    assert [model.code(n) for n in ("DIC2", "Alk2", "C")] == [A.PASSIVE(0), A.PASSIVE(1), A.PASSIVE(2)]
    assert model.G["DIC2"] is model.G["DIC1"]


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("mixed", 1e-5), ("f32", 5e-5)])
def test_oae_replicates_with_gas_exchange_and_release_match_oracle(precision, tol):
    g, bgc, model, vel, bcs, forcing = oae_model(precision)
    s0 = model.state_array().double().cpu().numpy()
    dt, nsteps = 300.0, 4
    obgc.time_step(model, dt, nsteps=nsteps)
    got = model.state_array().double().cpu().numpy()
    ref = oracle_run(model, bgc, g, vel, s0, dt, nsteps, bcs=bcs, forcing=forcing)
    errs = {n: rel_err(got[q], ref[q], floor_frac=FLOOR.get(n, 1e-6)) for q, n in enumerate(model.tracer_names)}
    worst = max(errs, key=errs.get)
    assert errs[worst] < tol, (worst, errs)
    # the release added alkalinity to Alk2 only (six stages fall inside [400, 1000) s: times 460,
    # 500, 600, 760, 800 and 900 of steps 1-3), so the excess of Alk2 over Alk1 grew
    q1, q2 = model.tracer_names.index("Alk1"), model.tracer_names.index("Alk2")
    excess_got = (got[q2] - got[q1]).sum() - (s0[q2] - s0[q1]).sum()
    excess_ref = (ref[q2] - ref[q1]).sum() - (s0[q2] - s0[q1]).sum()
    assert excess_ref > 0
    assert excess_got == pytest.approx(excess_ref, rel=max(tol, 1e-9) * 100)


def test_forcing_window_releases_its_integral():
    """Without gas exchange, Alk2 - Alk1 grows by the rate integrated over the stages of the window:
    a window over whole steps [t0, t0 + n dt) releases rate x n dt x cells (the RK3 stage weights of
    a step sum to one), whatever the advection does (periodic, conservative)."""
    g, bgc, model, vel, bcs, forcing = oae_model("f64", with_bcs=False, with_forcing=False)
    rate = np.zeros(g.shape)
    rate[-1, 4:9, 6:12] = 0.02
    model2 = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S", "C"), velocities=vel + (None,), precision="f64",
                                      forcing={"Alk2": obgc.Forcing(rate, start_time=300.0, end_time=900.0)})
    obgc.set_(model2, **{n: model.tracers[n] for n in model.tracer_names})
    s0 = model2.state_array().double().cpu().numpy()
    dt = 300.0
    obgc.time_step(model2, dt, nsteps=4)     # steps starting at 0, 300, 600, 900: two inside the window
    got = model2.state_array().double().cpu().numpy()
    q1, q2 = model2.tracer_names.index("Alk1"), model2.tracer_names.index("Alk2")
    released = (got[q2] - got[q1]).sum() - (s0[q2] - s0[q1]).sum()
    assert released == pytest.approx(rate.sum() * 2 * dt, rel=1e-10)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_replicates_without_conditions_track_each_other(precision):
    """DIC2 / Alk2 started equal to DIC1 / Alk1 evolve under the same tendency: they stay equal to
    rounding (the passive launch repeats the main launch's advection arithmetic)."""
    g, bgc, model, vel, bcs, forcing = oae_model(precision, with_bcs=False, with_forcing=False)
    obgc.set_(model, DIC2=model.tracers["DIC1"], Alk2=model.tracers["Alk1"])
    obgc.time_step(model, 300.0, nsteps=6)
    tol = 1e-13 if precision == "f64" else 1e-6
    for a, b in (("DIC1", "DIC2"), ("Alk1", "Alk2")):
        x, y = model.tracers[a].double().cpu().numpy(), model.tracers[b].double().cpu().numpy()
        assert rel_err(y, x) < tol


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("mixed", 1e-5)])
def test_zero_negative_tracers_reach_passive_tracers(precision, tol):
    mods = obgc.ZeroNegativeTracers(exclude=("Alk2",))
    # no gas exchange here: a negative Alk2 would make its pCO2 meaningless
    g, bgc, model, vel, bcs, forcing = oae_model(precision, with_bcs=False, with_forcing=False, modifiers=mods)
    obgc.set_(model, Alk2=-np.abs(model.tracers["Alk2"].double().cpu().numpy()))
    s0 = model.state_array().double().cpu().numpy()
    obgc.time_step(model, 300.0, nsteps=3)
    got = model.state_array().double().cpu().numpy()
    # the oracle's exclude mask is by slot (Alk2 is a passive slot there)
    names, src = oracle_layout(model)
    slot = {n: q for q, n in enumerate(model.tracer_names)}
    gas = [(bc.params, slot[name], slot[bc.water_concentration.DIC], slot[bc.water_concentration.Alk])
           for name, bc in bcs.items()]
    m = O.model3d(bgc.params, g.c_grid(), names, gas_exchange=gas, tendency_of=src, negatives=O.NEG_ZERO)
    m.zero_exclude_mask = 1 << slot["Alk2"]
    ref = np.ascontiguousarray(s0.copy())
    u, v = (x.double().cpu().numpy().ravel().copy() for x in vel)
    O.step3d(m, ref, u=u, v=v, t=0.0, dt=300.0, nsteps=3)
    errs = {n: rel_err(got[q], ref[q], floor_frac=FLOOR.get(n, 1e-6)) for q, n in enumerate(model.tracer_names)}
    worst = max(errs, key=errs.get)
    assert errs[worst] < tol, (worst, errs)
    C = got[model.tracer_names.index("C")]
    assert C.min() >= 0.0 and C.max() > 0.0                 # the passive tracer was zeroed where negative
    assert got[model.tracer_names.index("Alk2")].min() < 0  # the excluded one was not


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("mixed", 1e-5)])
def test_npzd_passive_tracers_with_diffusivity_match_oracle(precision, tol):
    # NonhydrostaticModel(; tracers = (:T, :C1, :C2, :C3), closure = ScalarDiffusivity(κ)) with NPZD:
    # three passive tracers (launches of 2 and 1) advected and diffused with the model's tracers,
    # one of them forced everywhere at a constant rate
    torch = cuda()
    g = obgc.RectilinearGrid((24, 16, 10), (4800.0, 3200.0, 100.0), dtype="f64")
    bgc = obgc.NPZD(g)
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=12)
    rate = np.full(g.shape, 1e-6)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "C1", "C2", "C3"), velocities=(u, v, None),
                                     precision=precision, closure=obgc.ScalarDiffusivity(κ=0.5),
                                     forcing={"C2": obgc.Forcing(rate)})
    rng = np.random.default_rng(12)
    obgc.set_(model, C1=rng.uniform(1, 2, g.shape), C2=rng.uniform(0.5, 1, g.shape), C3=rng.uniform(3, 4, g.shape))
    obgc.set_(model, N=7.0, P=0.1, Z=0.05, D=0.1, T=np.broadcast_to(np.linspace(8, 14, g.Nz)[:, None, None], g.shape))
    s0 = model.state_array().double().cpu().numpy()
    dt, nsteps = 120.0, 3
    obgc.time_step(model, dt, nsteps=nsteps)
    got = model.state_array().double().cpu().numpy()
    names, src = oracle_layout(model)
    slot = {n: q for q, n in enumerate(model.tracer_names)}
    m = O.model3d(bgc.params, g.c_grid(), names, kappa_h=0.5, kappa_z_faces=np.full(g.Nz + 1, 0.5), tendency_of=src,
                  forcing={slot["C2"]: (rate, -math.inf, math.inf)})
    ref = np.ascontiguousarray(s0.copy())
    uo, vo = (x.double().cpu().numpy().ravel().copy() for x in (u, v))
    O.step3d(m, ref, u=uo, v=vo, t=0.0, dt=dt, nsteps=nsteps)
    errs = {n: rel_err(got[q], ref[q]) for q, n in enumerate(model.tracer_names)}
    worst = max(errs, key=errs.get)
    assert errs[worst] < tol, (worst, errs)
    # the passive tracers kept their totals (periodic, no-flux walls), C2 gained rate x dt x cells
    for name, gain in (("C1", 0.0), ("C3", 0.0), ("C2", rate.sum() * dt * nsteps)):
        q = slot[name]
        assert got[q].sum() - s0[q].sum() == pytest.approx(gain, abs=(1e-9 if precision == "f64" else 1e-6) * s0[q].sum())


def test_oae_release_increases_co2_uptake():
    # examples/oae_experiment.jl in miniature: two identical carbonate systems, an alkalinity release
    # into the second; the added alkalinity lowers the surface pCO2, so the second system takes up
    # more CO2 from the air than the first (its DIC ends higher), while everything else stays equal
    torch = cuda()
    g, bgc, model, vel, bcs, forcing = oae_model("f64", with_forcing=False)
    obgc.set_(model, DIC2=model.tracers["DIC1"], Alk2=model.tracers["Alk1"])
    z, y, x = g.nodes()
    mask = ((x[None, None, :] - 2500) ** 2 + (y[None, :, None] - 2000) ** 2 < 1500.0 ** 2) & (z[:, None, None] > -4)
    release = obgc.Forcing(np.where(mask, 0.2, 0.0) * np.ones(g.shape), start_time=0.0, end_time=1800.0)
    oae = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S", "C"), velocities=vel + (None,),
                                   precision="f64", boundary_conditions=bcs, forcing={"Alk2": release})
    obgc.set_(oae, **{n: model.tracers[n] for n in model.tracer_names})
    obgc.time_step(oae, 300.0, nsteps=12)
    t = {n: oae.tracers[n].double().cpu().numpy() for n in oae.tracer_names}
    assert t["Alk2"].sum() > t["Alk1"].sum()
    assert t["DIC2"].sum() > t["DIC1"].sum()


def test_graph_replay_with_passive_launches_is_bit_identical():
    # obgc_step_graph captures the passive launches, the gas-exchange flux kernels and the clock
    # advance of the forcing windows with the main launch
    torch = cuda()
    runs = []
    for graph in (False, True):
        g, bgc, model, vel, bcs, forcing = oae_model("mixed", seed=8)
        obgc.time_step(model, 300.0, nsteps=5, graph=graph)
        runs.append(model.state_array().double().cpu().numpy())
    np.testing.assert_array_equal(runs[0], runs[1])


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("mixed", 1e-5)])
def test_forcing_of_a_model_tracer_with_implicit_diffusion_and_a_passive_tracer(precision, tol):
    # a forcing on NO3 (a tracer of the main launch) over a window that opens mid-step, a passive
    # tracer, and VerticallyImplicitTimeDiscretization acting on every slot after each stage
    torch = cuda()
    g = obgc.RectilinearGrid((36, 12, 10), (7200.0, 2400.0, 100.0), dtype="f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.05, seed=21)
    kz = np.linspace(1e-4, 0.3, g.Nz + 1)
    rate = np.zeros(g.shape)
    rate[-2:, 3:9, 5:20] = 5e-5
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S", "C"), velocities=(u, v, None),
                                     precision=precision, forcing={"NO3": obgc.Forcing(rate, start_time=250.0,
                                                                                        end_time=1000.0)})
    A.check(model._lib.obgc_set_diffusivity(model._ctx, 0.0, 0.0, (C.c_double * (g.Nz + 1))(*kz)),
            "obgc_set_diffusivity")
    A.check(model._lib.obgc_set_vertical_time_discretization(model._ctx, A.VERTICALLY_IMPLICIT), "vertical")
    rng = np.random.default_rng(21)
    obgc.set_(model, **obgc.lobster_initial_conditions(g, seed=22))
    obgc.set_(model, C=rng.uniform(1, 2, g.shape))
    s0 = model.state_array().double().cpu().numpy()
    dt, nsteps = 300.0, 4
    obgc.time_step(model, dt, nsteps=nsteps)
    got = model.state_array().double().cpu().numpy()
    names, src = oracle_layout(model)
    slot = {n: q for q, n in enumerate(model.tracer_names)}
    m = O.model3d(bgc.params, g.c_grid(), names, kappa_z_faces=kz, vertical_implicit=True, tendency_of=src,
                  forcing={slot["NO3"]: (rate, 250.0, 1000.0)})
    ref = np.ascontiguousarray(s0.copy())
    O.step3d(m, ref, u=u.double().cpu().numpy().ravel().copy(), v=v.double().cpu().numpy().ravel().copy(), t=0.0,
             dt=dt, nsteps=nsteps)
    errs = {n: rel_err(got[q], ref[q], floor_frac=FLOOR.get(n, 1e-6)) for q, n in enumerate(model.tracer_names)}
    worst = max(errs, key=errs.get)
    assert errs[worst] < tol, (worst, errs)
