"""Air-sea gas exchange on the GPU against the oracle: the flux of every column (constant and
per-column wind and air fields, FP64 and FP32 fields), and the fused 3-D step of LOBSTER with
carbonates and oxygen under CarbonDioxideGasExchangeBoundaryCondition on DIC and
OxygenGasExchangeBoundaryCondition on O2 (the reference's FieldBoundaryConditions(top = ...))."""
import numpy as np
import pytest

import obgc
import oracle as O
from obgc import _abi as A
from gpuhelp import cuda, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", ["f64", "f32"])
@pytest.mark.parametrize("gas", [A.GAS_CO2, A.GAS_O2])
def test_flux_of_every_column_matches_oracle(dtype, gas):
    torch = cuda()
    g = obgc.RectilinearGrid((13, 7, 5), (1300.0, 700.0, 50.0), dtype=dtype)
    td = torch.float32 if dtype == "f32" else torch.float64
    rng = np.random.default_rng(gas)
    host = dict(T=rng.uniform(0, 28, g.shape), S=rng.uniform(32, 37, g.shape), DIC=rng.uniform(1950, 2250, g.shape),
                Alk=rng.uniform(2250, 2450, g.shape), O2=rng.uniform(150, 330, g.shape))
    dev = {k: torch.as_tensor(v, dtype=td, device="cuda").contiguous() for k, v in host.items()}
    host = {k: v.double().cpu().numpy() for k, v in dev.items()}    # the values the kernel sees
    wind = torch.as_tensor(rng.uniform(0, 15, (g.Ny, g.Nx)), dtype=td, device="cuda")
    air = torch.as_tensor(rng.uniform(350, 500, (g.Ny, g.Nx)) if gas == A.GAS_CO2 else rng.uniform(8000, 10000, (g.Ny, g.Nx)),
                          dtype=td, device="cuda")
    ref_params = O.gas_exchange_defaults(gas)
    for fields in (False, True):
        bc = obgc.GasExchange(gas, wind_speed=wind if fields else 7.5, air_concentration=air if fields else None)
        out = bc.flux(g, dev["T"], dev["S"], DIC=dev["DIC"], Alk=dev["Alk"], O2=dev["O2"]).cpu().numpy()
        ref = np.zeros((g.Ny, g.Nx))
        w, a = wind.double().cpu().numpy(), air.double().cpu().numpy()
        for j in range(g.Ny):
            for i in range(g.Nx):
                s = (g.Nz - 1, j, i)
                ref[j, i] = O.gas_exchange_flux(ref_params, host["T"][s], host["S"][s], DIC=host["DIC"][s], Alk=host["Alk"][s],
                                                O2=host["O2"][s], u10=w[j, i] if fields else 7.5,
                                                air=a[j, i] if fields else ref_params.air_concentration)
        # CO2: the flux is the difference pCO2 - air, which amplifies the ~1e-13 relative rounding
        # differences of the pCO2 solve (exp vs pow forms of the constants, the Newton end point)
        assert rel_err(out, ref, floor_frac=1e-3) < 1e-10


def lobster_co_model(precision, shape=(24, 16, 10), seed=2):
    torch = cuda()
    g = obgc.RectilinearGrid(shape, (2400.0, 1600.0, 100.0), dtype="f32" if precision == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(), oxygen=obgc.Oxygen())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=seed)
    co2 = obgc.CarbonDioxideGasExchangeBoundaryCondition(wind_speed=10.0)
    o2 = obgc.OxygenGasExchangeBoundaryCondition(wind_speed=10.0)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=precision, boundary_conditions={"DIC": co2, "O2": o2})
    init = obgc.lobster_initial_conditions(g, seed=seed + 1)
    init["O2"] = 250.0
    obgc.set_(model, **{k: val for k, val in init.items() if k in model.tracers})
    return g, bgc, model, (u, v), (co2, o2)


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("mixed", 1e-5)])
def test_fused_step_with_gas_exchange_matches_oracle(precision, tol):
    g, bgc, model, vel, bcs = lobster_co_model(precision)
    s0 = model.state_array().double().cpu().numpy()
    dt, nsteps = 300.0, 4
    obgc.time_step(model, dt, nsteps=nsteps)
    got = model.state_array().double().cpu().numpy()
    m = O.model3d(bgc.params, g.c_grid(), model.tracer_names, gas_exchange=[b.params for b in bcs])
    ref = np.ascontiguousarray(s0.copy())
    u, v = (x.double().cpu().numpy().ravel().copy() for x in vel)
    O.step3d(m, ref, u=u, v=v, t=0.0, dt=dt, nsteps=nsteps)
    errs = {n: rel_err(got[q], ref[q]) for q, n in enumerate(model.tracer_names)}
    assert max(errs.values()) < tol, errs
    # the boundary conditions moved the surface DIC and O2 (by ~0.03 and ~1 mmol/m3 here), and
    # nothing below the surface level within these steps (no vertical velocity, neither sinks)
    m0 = O.model3d(bgc.params, g.c_grid(), model.tracer_names)
    ref0 = np.ascontiguousarray(s0.copy())
    O.step3d(m0, ref0, u=u, v=v, t=0.0, dt=dt, nsteps=nsteps)
    for name in ("DIC", "O2"):
        q = model.tracer_names.index(name)
        assert np.max(np.abs(ref[q, -1] - ref0[q, -1])) > 1e-3
        assert np.max(np.abs(got[q, -1] - ref0[q, -1])) > 1e-3
        assert np.array_equal(ref[q, :-1], ref0[q, :-1])
