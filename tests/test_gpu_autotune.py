"""The fused step's launch-shape autotuner (obgc_autotune_step): it leaves the caller's state as it
found it (tracers, gas-exchange warm starts, sediment storage), keeps one of its candidates, and the
steps after it equal those of a model set to the same shape by hand (and the oracle)."""
import numpy as np
import pytest

import obgc
import oracle as O
from obgc import _abi as A
from gpuhelp import cuda, rel_err

pytestmark = pytest.mark.gpu

CANDIDATES = {2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 16, 24, 32}


def lobster(precision, shape, seed=3, gas=False):
    cuda()
    g = obgc.RectilinearGrid(shape, (100.0 * shape[0], 100.0 * shape[1], 10.0 * shape[2]),
                             dtype="f32" if precision == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(), oxygen=obgc.Oxygen() if gas else None)
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=seed)
    bcs = {}
    if gas:
        bcs = {"DIC": obgc.CarbonDioxideGasExchangeBoundaryCondition(wind_speed=10.0),
               "O2": obgc.OxygenGasExchangeBoundaryCondition(wind_speed=10.0)}
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=precision, boundary_conditions=bcs)
    init = obgc.lobster_initial_conditions(g, seed=seed + 1)
    if gas:
        init["O2"] = 250.0
    obgc.set_(model, **{k: val for k, val in init.items() if k in model.tracers})
    return g, bgc, model, (u, v), bcs


@pytest.mark.parametrize("precision,shape,gas", [("f32", (64, 48, 20), False), ("f64", (24, 16, 10), True)])
def test_autotune_keeps_the_state_and_a_candidate(precision, shape, gas):
    g, bgc, model, vel, bcs = lobster(precision, shape, gas=gas)
    dt = 300.0
    if gas:
        obgc.time_step(model, dt, nsteps=2)          # the gas exchange's [H+] warm starts exist
    s0 = model.state_array().clone()
    t0 = model.clock.time
    tz, staging, ms = model.autotune(dt, steps=2)
    assert model.clock.time == t0
    assert bool((model.state_array() == s0).all())   # bit for bit
    assert tz in {min(c, g.Nz) for c in CANDIDATES}
    assert staging in (0, 1) and (staging == 0 or model.staging()[0])
    assert ms > 0

    # the steps after the autotuner equal a model set to the same shape by hand (its warm starts
    # from the same two steps), and the oracle
    _, _, twin, _, _ = lobster(precision, shape, gas=gas)
    if gas:
        obgc.time_step(twin, dt, nsteps=2)
    twin.set_tiling(tz)
    twin.set_staging(staging)
    obgc.time_step(model, dt, nsteps=3)
    obgc.time_step(twin, dt, nsteps=3)
    got = model.state_array().double().cpu().numpy()
    assert np.array_equal(got, twin.state_array().double().cpu().numpy())
    m = O.model3d(bgc.params, g.c_grid(), model.tracer_names,
                  gas_exchange=[b.params for b in bcs.values()] if gas else ())
    ref = np.ascontiguousarray(s0.double().cpu().numpy())
    u, v = (x.double().cpu().numpy().ravel().copy() for x in vel)
    O.step3d(m, ref, u=u, v=v, t=t0, dt=dt, nsteps=3)
    tol = {"f64": 1e-10, "f32": 5e-5}[precision]
    assert max(rel_err(got[q], ref[q]) for q in range(got.shape[0])) < tol


def test_autotune_keeps_the_sediment_storage():
    cuda()
    g = obgc.RectilinearGrid((8, 8, 20), (800.0, 800.0, 200.0), ("Periodic", "Periodic", "Bounded"), dtype="f64")
    sed = obgc.InstantRemineralisationSediment(g, sinking_tracers=("sPOM", "bPOM"), remineralisation_reciever="NH4")
    bgc = obgc.LOBSTER(g, sediment=sed)
    bgc.params.open_bottom = 1
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, precision="f64")
    obgc.set_(model, NO3=10.0, NH4=0.5, P=0.5, Z=0.1, sPOM=1.0, bPOM=1.0, DOM=0.1)
    obgc.time_step(model, 300.0, nsteps=4)
    s0, st0 = model.state_array().clone(), model.sediment_storage().copy()
    model.autotune(300.0, steps=2)
    assert bool((model.state_array() == s0).all())
    assert np.array_equal(model.sediment_storage(), st0)


def test_autotune_rejects_bad_arguments():
    _, _, model, _, _ = lobster("f64", (16, 16, 8))
    with pytest.raises(A.ObgcError):
        model.autotune(-1.0)
    with pytest.raises(A.ObgcError):
        model.autotune(300.0, steps=0)
