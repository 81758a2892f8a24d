"""SimpleMultiGSediment under the fused 3-D step against the oracle: LOBSTER + Oxygen with sinking
detritus through an open bottom, the sediment's fields and the water tracers after 12 steps (FP64
1e-11, mixed 1e-5), and the same first-order nitrogen budget as the oracle's."""
import numpy as np
import pytest

import obgc
import oracle as O
from gpuhelp import cuda, rel_err
from test_oracle_multig import NAMES, default_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("f64", 1e-11), ("mixed", 1e-5)])
def test_multig_sediment_matches_oracle(precision, tol):
    torch = cuda()
    g = obgc.RectilinearGrid((16, 8, 12), (1600.0, 800.0, 120.0), ("Periodic", "Periodic", "Bounded"), dtype="f64")
    sed = obgc.SimpleMultiGSediment(g)
    bgc = obgc.LOBSTER(g, oxygen=obgc.Oxygen(), sediment=sed)
    bgc.params.open_bottom = 1
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.05, seed=9)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, velocities=(u, v, None), precision=precision)
    assert list(model.tracer_names) == NAMES
    rng = np.random.default_rng(3)
    init = dict(NO3=10.0, NH4=0.5, P=0.5, Z=0.1, sPOM=1.0, bPOM=1.0, DOM=0.1, O2=250.0)
    init = {n: x * np.exp(0.1 * rng.standard_normal(g.shape)) for n, x in init.items()}
    obgc.set_(model, **init)
    s0 = model.state_array().double().cpu().numpy()
    dt, nsteps = 600.0, 12
    obgc.time_step(model, dt, nsteps=nsteps)
    got = model.state_array().double().cpu().numpy()
    fields = model.sediment_fields()

    ref = np.ascontiguousarray(s0.copy())
    m = O.model3d(bgc.params, g.c_grid(), NAMES)
    ref_sed = O.attach_multig(m, sed.params, NAMES, sed.sinking_nitrogen, g)
    O.step3d(m, ref, u=u.cpu().numpy().ravel().copy(), v=v.cpu().numpy().ravel().copy(), t=0.0, dt=dt, nsteps=nsteps)
    NN = g.Nx * g.Ny
    errs = {n: rel_err(got[q], ref[q]) for q, n in enumerate(NAMES)}
    assert max(errs.values()) < tol, errs
    ref_fields = ref_sed[:3 * NN].reshape(3, g.Ny, g.Nx)
    for q in range(3):
        assert rel_err(fields[q], ref_fields[q]) < tol, q
    assert np.all(fields > 0)
    # a second call continues the sediment's clock (no fresh first tendency): 1 + 11 steps = 12
    model2 = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, velocities=(u, v, None), precision=precision)
    obgc.set_(model2, **init)
    obgc.time_step(model2, dt, nsteps=1)
    obgc.time_step(model2, dt, nsteps=nsteps - 1)
    assert rel_err(model2.sediment_fields(), fields) < (1e-13 if precision == "f64" else 1e-6)
