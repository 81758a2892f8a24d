"""The fused step's device-side status word: a NaN written into the state and an unconverged surface
pCO2 solve are reported by obgc_step (status check on, the default) and by obgc_step_status after
obgc_step_graph.  Both failures are made on the host (a NaN in the input; an alkalinity whose [H+]
lies below the bisection guard's range, with the Newton iterations capped at one); no kernel
faults, and every later call on the context still works."""
import math

import numpy as np
import pytest

import obgc
from obgc import _abi as A
from gpuhelp import cuda

pytestmark = pytest.mark.gpu


def lobster(precision, gas=False, shape=(16, 16, 8), max_iters=100):
    cuda()
    g = obgc.RectilinearGrid(shape, (1600.0, 1600.0, 80.0), dtype="f32" if precision == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=3)
    cc = obgc.CarbonChemistry(max_iters=max_iters)
    bcs = {"DIC": obgc.CarbonDioxideGasExchangeBoundaryCondition(wind_speed=10.0, carbon_chemistry=cc)} if gas else None
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=precision, boundary_conditions=bcs)
    init = obgc.lobster_initial_conditions(g, seed=4)
    obgc.set_(model, **init)
    return model, init


def raw_step(model, graph=False):
    fn = model._lib.obgc_step_graph if graph else model._lib.obgc_step
    return fn(model._ctx, model.clock.time, 300.0, 2, model._stream())


@pytest.mark.parametrize("precision,bad", [("f32", math.nan), ("mixed", math.nan), ("f64", math.nan),
                                          ("f32", math.inf), ("f64", -math.inf)])
def test_nan_in_the_state_is_reported(precision, bad):
    model, init = lobster(precision)
    p = model.tracers["P"].cpu().numpy().copy()
    p[3, 4, 5] = bad
    obgc.set_(model, P=p)
    with pytest.raises(A.ObgcError) as e:
        obgc.time_step(model, 300.0, nsteps=2)
    assert e.value.status == A.ERR_NAN
    assert "NaN" in A.load().obgc_last_error_message().decode()
    # without the check the call returns at once; the flag waits in the status word
    model.set_status_check(False)
    assert raw_step(model) == A.OBGC_OK
    rc, flags = model.step_status()
    assert rc == A.ERR_NAN and flags & A.FLAG_NAN
    # graph replay: the same flag through obgc_step_status
    assert raw_step(model, graph=True) == A.OBGC_OK
    rc, flags = model.step_status()
    assert rc == A.ERR_NAN and flags & A.FLAG_NAN
    # a clean state: the word is cleared by every call
    obgc.set_(model, **init)
    model.set_status_check(True)
    obgc.time_step(model, 300.0, nsteps=2)
    assert model.step_status() == (A.OBGC_OK, 0)
    assert raw_step(model, graph=True) == A.OBGC_OK
    assert model.step_status() == (A.OBGC_OK, 0)
    assert np.all(np.isfinite(model.state_array().cpu().numpy()))


@pytest.mark.parametrize("precision", ["f32", "mixed"])
def test_unconverged_surface_pco2_solve_is_reported(precision):
    """At an alkalinity of 1e9 umol/kg the residual's root is [H+] ~ 1e-17 (Kw / Alk), below the
    bisection guard's range [1e-14, 1]: with one Newton iteration allowed the solve ends unconverged
    in that surface cell (every other cell converges through the guard)."""
    model, init = lobster(precision, gas=True, max_iters=1)
    alk = model.tracers["Alk"].cpu().numpy().copy()
    alk[-1, 2, 3] = 1e9
    obgc.set_(model, Alk=alk)
    model.set_status_check(False)
    assert raw_step(model) == A.OBGC_OK
    rc, flags = model.step_status()
    assert flags & A.FLAG_NOT_CONVERGED
    assert rc == (A.ERR_NAN if flags & A.FLAG_NAN else A.ERR_NOT_CONVERGED)
    model.set_status_check(True)
    with pytest.raises(A.ObgcError) as e:
        obgc.time_step(model, 300.0, nsteps=1)
    assert e.value.status in (A.ERR_NOT_CONVERGED, A.ERR_NAN)
    # the ordinary surface: every solve converges
    obgc.set_(model, **init)
    obgc.time_step(model, 300.0, nsteps=2)
    assert model.step_status() == (A.OBGC_OK, 0)
