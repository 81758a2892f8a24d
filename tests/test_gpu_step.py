"""GPU parity of the fused 3-D RK3 step (WENO5 advection + drift + BGC + TwoBand PAR + RK3)
against the oracle on seeded inputs, in FP64, FP32 and mixed precision, plus conservation,
graph replay, halo'd layouts and the compensated budget."""
import math

import numpy as np
import pytest

import obgc
import oracle as O
from gpuhelp import cuda, rel_err

pytestmark = pytest.mark.gpu


def lobster_model(shape=(40, 24, 12), extent=(4000.0, 2400.0, 120.0), precision="f64", topo=("Periodic", "Periodic", "Bounded"),
                  seed=1, carbonates=True, TZ=None, open_bottom=True, w=False):
    torch = cuda()
    g = obgc.RectilinearGrid(shape, extent, topo, dtype="f32" if precision == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem() if carbonates else None)
    bgc.params.open_bottom = int(open_bottom)
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=seed)
    wv = None
    if w:
        rng = np.random.default_rng(seed + 7)
        wv = torch.as_tensor(rng.normal(0, 1e-4, g.shape), dtype=torch.float64, device="cuda")
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S") if carbonates else (),
                                     velocities=(u, v, wv), precision=precision)
    if TZ:
        model.set_tiling(TZ)
    init = obgc.lobster_initial_conditions(g, seed=seed + 1)
    obgc.set_(model, **{k: v for k, v in init.items() if k in model.tracers})
    return g, bgc, model, (u, v, wv)


def oracle_run(g, bgc, model, vel, state0, dt, nsteps, t0=0.0):
    m = O.model3d(bgc.params, g.c_grid(), model.tracer_names)
    ref = np.ascontiguousarray(state0.astype(np.float64))
    u, v, w = (None if x is None else x.double().cpu().numpy().ravel().copy() for x in vel)
    O.step3d(m, ref, u=u, v=v, w=w, t=t0, dt=dt, nsteps=nsteps)
    return ref


def per_tracer_err(model, got, ref):
    return {n: rel_err(got[q], ref[q]) for q, n in enumerate(model.tracer_names)}


@pytest.mark.parametrize("TZ", [None, 5])
def test_fused_fp64_matches_oracle(TZ):
    g, bgc, model, vel = lobster_model(TZ=TZ)
    s0 = model.state_array().cpu().numpy()
    obgc.time_step(model, 300.0, nsteps=4)
    got = model.state_array().cpu().numpy()
    ref = oracle_run(g, bgc, model, vel, s0, 300.0, 4)
    errs = per_tracer_err(model, got, ref)
    assert max(errs.values()) < 1e-11, errs
    assert np.max(np.abs(got - s0)) > 0


@pytest.mark.parametrize("precision,tol", [("mixed", 1e-5), ("f32", 5e-5)])
def test_fused_f32_and_mixed_within_tolerance(precision, tol):
    # mixed (FP64 state, FP32 arithmetic) carries the path's 1e-5 statement; the FP32-state path
    # loses up to ~1e-5 on tracers that grow from zero (sPOM) within a few steps
    if True:
        g, bgc, model, vel = lobster_model(precision=precision, seed=4)
        s0 = model.state_array().double().cpu().numpy()
        obgc.time_step(model, 300.0, nsteps=6)
        got = model.state_array().double().cpu().numpy()
        ref = oracle_run(g, bgc, model, vel, s0, 300.0, 6)
        errs = per_tracer_err(model, got, ref)
        assert max(errs.values()) < tol, (precision, errs)


@pytest.mark.parametrize("topo", [("Bounded", "Periodic", "Bounded"), ("Periodic", "Bounded", "Bounded")])
def test_f32_full_and_ragged_tiles(topo):
    # FP32 on a grid of two full-width tiles and a ragged one in x, with walls in x or in y
    g, bgc, model, vel = lobster_model(shape=(72, 20, 10), extent=(7200.0, 2000.0, 100.0), precision="f32", topo=topo,
                                       seed=6)
    s0 = model.state_array().double().cpu().numpy()
    # dt = 150 s: the test flow (0.34 m/s at most across 100 m cells) stays below CFL 0.7
    obgc.time_step(model, 150.0, nsteps=4)
    got = model.state_array().double().cpu().numpy()
    ref = oracle_run(g, bgc, model, vel, s0, 150.0, 4)
    errs = per_tracer_err(model, got, ref)
    assert max(errs.values()) < 5e-5, errs


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("mixed", 1e-5)])
def test_vertically_implicit_diffusivity_matches_oracle(precision, tol):
    # VerticalScalarDiffusivity(VerticallyImplicitTimeDiscretization(), κ = κ(z)) with a 0.5 m2/s
    # mixed layer over 10 m cells at dt = 600 s (dt κ / dz^2 = 3: far beyond an explicit step), and
    # scale_negatives = true, which then runs after the implicit solve of every stage
    torch = cuda()
    g = obgc.RectilinearGrid((40, 16, 12), (8000.0, 3200.0, 120.0), dtype="f32" if precision == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(), scale_negatives=True)
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.05, seed=3)
    kz = lambda z: 0.5 * (1 + math.tanh((z + 50.0) / 10.0)) / 2 + 1e-4   # noqa: E731
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=precision,
                                     closure=obgc.VerticalScalarDiffusivity(obgc.VerticallyImplicitTimeDiscretization(), κ=kz))
    obgc.set_(model, **obgc.lobster_initial_conditions(g, seed=5))
    s0 = model.state_array().double().cpu().numpy()
    dt, nsteps = 600.0, 4
    obgc.time_step(model, dt, nsteps=nsteps)
    got = model.state_array().double().cpu().numpy()
    zf = -g.Lz + g.Lz / g.Nz * np.arange(g.Nz + 1)
    m = O.model3d(bgc.params, g.c_grid(), model.tracer_names, kappa_z_faces=np.array([kz(z) for z in zf]),
                  vertical_implicit=True, negatives=O.NEG_SCALE)
    ref = np.ascontiguousarray(s0.copy())
    O.step3d(m, ref, u=u.double().cpu().numpy().ravel().copy(), v=v.double().cpu().numpy().ravel().copy(), t=0.0,
             dt=dt, nsteps=nsteps)
    errs = per_tracer_err(model, got, ref)
    assert max(errs.values()) < tol, errs
    # the mixed layer homogenised T (a linear profile at the start)
    q = model.tracer_names.index("T")
    top = got[q, -4:]
    assert np.ptp(top) < 0.2 * np.ptp(s0[q, -4:])


def test_bounded_walls_vertical_velocity_and_sinking():
    g, bgc, model, vel = lobster_model(shape=(21, 13, 17), extent=(2100.0, 1300.0, 170.0),
                                       topo=("Bounded", "Bounded", "Bounded"), w=True, carbonates=False, seed=8)
    s0 = model.state_array().cpu().numpy()
    obgc.time_step(model, 200.0, nsteps=3)
    got = model.state_array().cpu().numpy()
    ref = oracle_run(g, bgc, model, vel, s0, 200.0, 3)
    assert max(per_tracer_err(model, got, ref).values()) < 1e-11


def test_npzd_front_2d_fp64():
    torch = cuda()
    g = obgc.RectilinearGrid((160, 32), (10000.0, 500.0), ("Bounded", "Flat", "Bounded"))
    bgc = obgc.NPZD(g)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, precision="f64")
    obgc.set_(model, **obgc.npzd_front_initial_conditions(g))
    s0 = model.state_array().cpu().numpy()
    obgc.time_step(model, 50.0, nsteps=20)
    got = model.state_array().cpu().numpy()
    ref = oracle_run(g, bgc, model, (None, None, None), s0, 50.0, 20)
    assert max(per_tracer_err(model, got, ref).values()) < 1e-11


def test_nitrogen_and_carbon_conserved_closed_bottom():
    g, bgc, model, vel = lobster_model(open_bottom=False, seed=12)
    N0, C0 = model.budget("nitrogen"), model.budget("carbon")
    obgc.time_step(model, 300.0, nsteps=10)
    N1, C1 = model.budget("nitrogen"), model.budget("carbon")
    assert abs(N1 - N0) / N0 < 1e-12
    assert abs(C1 - C0) / C0 < 1e-12


def test_budget_is_compensated_sum():
    torch = cuda()
    g, bgc, model, vel = lobster_model(seed=13)
    got = model.budget("nitrogen")
    names = obgc.conserved_tracers(bgc, labeled=True)["nitrogen"]
    ref = math.fsum(float(x) for n in names for x in model.tracers[n].cpu().numpy().ravel())
    assert abs(got - ref) <= 1e-15 * abs(ref)


def test_graph_replay_and_odd_steps_are_bitwise_identical():
    torch = cuda()
    _, _, a, _ = lobster_model(precision="f32", seed=21)
    _, _, b, _ = lobster_model(precision="f32", seed=21)
    obgc.time_step(a, 300.0, nsteps=3)
    obgc.time_step(b, 300.0, nsteps=3, graph=True)
    torch.cuda.synchronize()
    assert torch.equal(a.state_array(), b.state_array())
    obgc.time_step(a, 300.0, nsteps=2)
    obgc.time_step(b, 300.0, nsteps=1)
    obgc.time_step(b, 300.0, nsteps=1)
    torch.cuda.synchronize()
    assert torch.equal(a.state_array(), b.state_array())


@pytest.mark.parametrize("precision", ["f32", "f64"])
def test_zero_state_stays_zero(precision):
    # test_NutrientsPlanktonDetritus.jl:101-112: a zero state stays exactly zero (the eps(0.0)
    # guards must turn 0/0 into 0), here through advection, sinking, light and RK3
    torch = cuda()
    g = obgc.RectilinearGrid((40, 16, 12), (4000.0, 1600.0, 120.0), dtype="f32" if precision == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=2)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=precision)
    obgc.time_step(model, 300.0, nsteps=3)
    torch.cuda.synchronize()
    assert torch.count_nonzero(model.state_array()).item() == 0


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("mixed", 1e-5)])
def test_fused_step_with_scalar_diffusivity_matches_oracle(precision, tol):
    # closure = HorizontalScalarDiffusivity(κ = 5 m2/s), VerticalScalarDiffusivity(κ(z)) with a
    # mixed-layer profile through the faces, and an isotropic ScalarDiffusivity(κ = 0.05 m2/s), all
    # explicit (stable at these steps), with Bounded x walls (no flux) and periodic y
    torch = cuda()
    g = obgc.RectilinearGrid((24, 16, 12), (2400.0, 1600.0, 120.0), ("Bounded", "Periodic", "Bounded"),
                             dtype="f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    # a divergence-free shear flow: no x velocity (Bounded walls), v varying with x only
    u = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    xc = (np.arange(g.Nx) + 0.5) / g.Nx
    v = torch.as_tensor(np.broadcast_to(0.05 * np.sin(2 * np.pi * xc), g.shape).copy(), dtype=torch.float64,
                        device="cuda")
    kz = lambda z: 1e-2 * (1 + math.tanh((z + 40.0) / 10.0)) / 2 + 1e-4   # noqa: E731
    zf = -g.Lz + g.Lz / g.Nz * np.arange(g.Nz + 1)
    cases = [(obgc.HorizontalScalarDiffusivity(κ=5.0), 5.0, None),
             (obgc.VerticalScalarDiffusivity(κ=kz), 0.0, np.array([kz(z) for z in zf])),
             (obgc.ScalarDiffusivity(κ=0.05), 0.05, np.full(g.Nz + 1, 0.05))]
    init = obgc.lobster_initial_conditions(g, seed=9)
    uo, vo = (x.double().cpu().numpy().ravel().copy() for x in (u, v))
    dt, nsteps = 200.0, 3
    for closure, kh, kzf in cases:
        mdl = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                       precision=precision, closure=closure)
        obgc.set_(mdl, **init)
        s0 = mdl.state_array().double().cpu().numpy()
        obgc.time_step(mdl, dt, nsteps=nsteps)
        got = mdl.state_array().double().cpu().numpy()
        m = O.model3d(bgc.params, g.c_grid(), mdl.tracer_names, kappa_h=kh, kappa_z_faces=kzf)
        ref = np.ascontiguousarray(s0.copy())
        O.step3d(m, ref, u=uo, v=vo, t=0.0, dt=dt, nsteps=nsteps)
        errs = per_tracer_err(mdl, got, ref)
        assert max(errs.values()) < tol, errs
        # diffusion moved the state: the same run without a closure differs by far more than the tolerance
        m0 = O.model3d(bgc.params, g.c_grid(), mdl.tracer_names)
        ref0 = np.ascontiguousarray(s0.copy())
        O.step3d(m0, ref0, u=uo, v=vo, t=0.0, dt=dt, nsteps=nsteps)
        assert max(per_tracer_err(mdl, ref0, ref).values()) > 100 * tol


@pytest.mark.parametrize("base,precision,tol", [("NPZD", "f64", 1e-11), ("LOBSTER", "f64", 1e-11),
                                                ("LOBSTER", "mixed", 1e-5)])
def test_instant_remineralisation_sediment(base, precision, tol):
    # InstantRemineralisationSediment: the GPU step against the oracle (tracers and storage), and
    # nitrogen conserved between the water and the sediment (the reference's
    # test/test_sediments.jl:58-80 statement), with an open bottom
    torch = cuda()
    g = obgc.RectilinearGrid((8, 8, 20), (800.0, 800.0, 200.0), ("Periodic", "Periodic", "Bounded"), dtype="f64")
    if base == "NPZD":
        sed = obgc.InstantRemineralisationSediment(g)
        bgc = obgc.NPZD(g, sediment=sed)
        init = dict(N=10.0, P=0.5, Z=0.1, D=1.0, T=12.0)
    else:
        sed = obgc.InstantRemineralisationSediment(g, sinking_tracers=("sPOM", "bPOM"), remineralisation_reciever="NH4")
        bgc = obgc.LOBSTER(g, sediment=sed)
        init = dict(NO3=10.0, NH4=0.5, P=0.5, Z=0.1, sPOM=1.0, bPOM=1.0, DOM=0.1)
    bgc.params.open_bottom = 1
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, precision=precision)   # no velocity: sinking only
    obgc.set_(model, **{k: v for k, v in init.items() if k in model.tracers})
    s0 = model.state_array().double().cpu().numpy()
    dt, nsteps = 300.0, 12
    obgc.time_step(model, dt, nsteps=nsteps)
    got = model.state_array().double().cpu().numpy()
    storage = model.sediment_storage()
    ref = np.ascontiguousarray(s0.copy())
    ref_storage = np.zeros((g.Ny, g.Nx))
    m = O.model3d(bgc.params, g.c_grid(), model.tracer_names,
                  sediment=(sed.sinking_tracers, sed.remineralisation_reciever, sed.a, sed.b, sed.k, ref_storage))
    O.step3d(m, ref, t=0.0, dt=dt, nsteps=nsteps)
    errs = per_tracer_err(model, got, ref)
    assert max(errs.values()) < tol, errs
    assert rel_err(storage, ref_storage) < tol
    assert np.all(storage > 0)
    # nitrogen: the volume integral of the tracers' nitrogen plus the area integral of the storage
    names = obgc.conserved_tracers(bgc, labeled=True)["nitrogen"]
    dV, dA = g.Lx * g.Ly * g.Lz / g.N, g.Lx * g.Ly / (g.Nx * g.Ny)
    def total(state, st):
        return sum(state[model.tracer_names.index(n)].sum() for n in names) * dV + st.sum() * dA
    n0 = total(s0, np.zeros_like(storage))
    assert abs(total(got, storage) - n0) / n0 < (1e-13 if precision == "f64" else 1e-6)


@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("mixed", 1e-5)])
def test_eady_like_configuration_matches_oracle(precision, tol):
    # the options of the reference's Eady example together (examples/eady.jl:50-73): LOBSTER with
    # carbonates and scale_negatives, T and S, VerticalScalarDiffusivity(κ = 1e-4), and the CO2
    # gas exchange on DIC, with a random-streamfunction flow
    torch = cuda()
    g = obgc.RectilinearGrid((32, 16, 12), (3200.0, 1600.0, 60.0), ("Periodic", "Periodic", "Bounded"), dtype="f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(), scale_negatives=True)
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=21)
    co2 = obgc.CarbonDioxideGasExchangeBoundaryCondition(wind_speed=8.0)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=precision, closure=obgc.VerticalScalarDiffusivity(κ=1e-4),
                                     boundary_conditions={"DIC": co2})
    init = obgc.lobster_initial_conditions(g, seed=22)
    init["NH4"] = np.random.default_rng(23).normal(0.0, 0.05, g.shape)   # negatives to scale away
    obgc.set_(model, **{k: val for k, val in init.items() if k in model.tracers})
    s0 = model.state_array().double().cpu().numpy()
    dt, nsteps = 200.0, 4
    obgc.time_step(model, dt, nsteps=nsteps, graph=True)
    got = model.state_array().double().cpu().numpy()
    m = O.model3d(bgc.params, g.c_grid(), model.tracer_names, negatives=O.NEG_SCALE, gas_exchange=[co2.params],
                  kappa_z_faces=np.full(g.Nz + 1, 1e-4))
    ref = np.ascontiguousarray(s0.copy())
    O.step3d(m, ref, u=u.double().cpu().numpy().ravel().copy(), v=v.double().cpu().numpy().ravel().copy(),
             t=0.0, dt=dt, nsteps=nsteps)
    errs = {n: rel_err(got[q], ref[q], floor_frac=1e-3) for q, n in enumerate(model.tracer_names)}
    assert max(errs.values()) < tol, errs
    assert np.min(got[model.tracer_names.index("NH4")]) >= 0
