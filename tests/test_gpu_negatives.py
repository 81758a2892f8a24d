"""Negative-tracer modifiers on the GPU: the reference's known answers (test/test_utils.jl:7-40)
through the 3-D model, the standalone kernels against the oracle, and the 3-D fused step and the
column engine with scale_negatives = true against the oracle."""
import math

import numpy as np
import pytest

import obgc
import oracle as O
from gpuhelp import cuda, rel_err

pytestmark = pytest.mark.gpu


def one_cell_model(bgc, precision="f64"):
    g = obgc.RectilinearGrid((1, 1, 1), (1.0, 1.0, 1.0), dtype="f32" if precision == "f32" else "f64")
    return obgc.NonhydrostaticModel(g, biogeochemistry=bgc, precision=precision)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_scale_negatives_known_answer(precision):
    cuda()
    g = obgc.RectilinearGrid((1, 1, 1), (1.0, 1.0, 1.0))
    model = one_cell_model(obgc.NPZD(g, scale_negatives=True), precision)
    obgc.set_(model, N=2.0, P=-1.0)
    obgc.time_step(model, 1e-10, nsteps=1)
    N = float(model.tracers["N"].cpu()[0, 0, 0])
    P = float(model.tracers["P"].cpu()[0, 0, 0])
    assert N == pytest.approx(1.0, rel=1e-6) and P == pytest.approx(0.0, abs=1e-6)


def test_zero_negatives_known_answer():
    cuda()
    g = obgc.RectilinearGrid((1, 1, 1), (1.0, 1.0, 1.0))
    model = one_cell_model(obgc.NPZD(g, modifiers=obgc.ZeroNegativeTracers(exclude=("Z",))))
    obgc.set_(model, N=2.0, P=-1.0, Z=-1.0)
    obgc.time_step(model, 1e-10, nsteps=1)
    out = {n: float(model.tracers[n].cpu()[0, 0, 0]) for n in ("N", "P", "Z")}
    assert out["N"] == pytest.approx(2.0, rel=1e-8)
    assert out["P"] == pytest.approx(0.0, abs=1e-8)
    assert out["Z"] == pytest.approx(-1.0, rel=1e-6)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_scale_negatives_kernel_matches_oracle(dtype):
    torch = cuda()
    g = obgc.RectilinearGrid((37, 19, 11), (1.0, 1.0, 1.0), dtype=dtype)
    rng = np.random.default_rng(2)
    names = ("P", "Z", "DIC", "sPOM", "bPOM", "DOM")
    host = {n: rng.normal(0.3, 1.0, g.shape) for n in names}
    host["DIC"] = rng.normal(1.0, 3.0, g.shape)
    host["P"].flat[5] = math.nan
    td = torch.float32 if dtype == "f32" else torch.float64
    dev = {n: torch.as_tensor(v, dtype=td, device="cuda") for n, v in host.items()}
    sf = (7.3, 6.56, 1.0, 6.56, 6.56, 6.56)
    obgc.ScaleNegativeTracers(names, scalefactors=sf, invalid_fill_value=0.5).apply(dev, g)
    torch.cuda.synchronize()
    npdt = np.float32 if dtype == "f32" else np.float64
    ref = [np.ascontiguousarray(host[n].astype(npdt).astype(np.float64).ravel()) for n in names]
    O.scale_negatives(ref, sf, 0.5)
    for q, n in enumerate(names):
        got = dev[n].double().cpu().numpy().ravel()
        if dtype == "f64":
            np.testing.assert_array_equal(got, ref[q])      # same operations, same rounding
        else:
            np.testing.assert_allclose(got, ref[q].astype(np.float32).astype(np.float64), rtol=2e-7, atol=1e-30,
                                       equal_nan=True)
    assert not any(np.nanmin(dev[n].cpu().numpy()) < 0 for n in names)


@pytest.mark.parametrize("mode,precision,tol", [("scale", "f64", 1e-10), ("scale", "mixed", 1e-5),
                                                ("zero", "f64", 1e-10)])
def test_fused_step_with_scale_negatives_matches_oracle(mode, precision, tol):
    # the modifier runs inside the substep's update (after every substep), as update_state! does
    torch = cuda()
    g = obgc.RectilinearGrid((24, 16, 10), (2400.0, 1600.0, 100.0), ("Periodic", "Periodic", "Bounded"),
                             dtype="f64")
    if mode == "scale":
        bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(), scale_negatives=True)
    else:
        bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(),
                           modifiers=obgc.ZeroNegativeTracers(exclude=("DOM",)))
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=4)
    model = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=precision)
    init = obgc.lobster_initial_conditions(g, seed=5)
    rng = np.random.default_rng(9)
    init["NH4"] = rng.normal(0.0, 0.05, g.shape)      # negatives to be scaled away
    init["DOM"] = rng.normal(0.0, 0.02, g.shape)
    obgc.set_(model, **{k: v for k, v in init.items() if k in model.tracers})
    s0 = model.state_array().cpu().numpy()
    obgc.time_step(model, 200.0, nsteps=3)
    got = model.state_array().cpu().numpy()
    m = O.model3d(bgc.params, g.c_grid(), model.tracer_names, negatives=O.NEG_SCALE if mode == "scale" else O.NEG_ZERO,
                  zero_exclude=("DOM",) if mode == "zero" else ())
    ref = np.ascontiguousarray(s0.astype(np.float64))
    O.step3d(m, ref, u=u.double().cpu().numpy().ravel().copy(), v=v.double().cpu().numpy().ravel().copy(),
             t=0.0, dt=200.0, nsteps=3)
    nh4 = model.tracer_names.index("NH4")
    assert np.min(got[nh4]) >= 0 and np.min(s0[nh4]) < 0
    if mode == "zero":
        assert np.min(got[model.tracer_names.index("DOM")]) < 0      # excluded from zeroing
    errs = {n: rel_err(got[q], ref[q], floor_frac=1e-3) for q, n in enumerate(model.tracer_names)}
    assert max(errs.values()) < tol, errs


@pytest.mark.parametrize("precision,eps,floor", [("f64", 2.0 ** -53, 1e-12), ("f32", 2.0 ** -24, 1e-4),
                                                 ("mixed", 2.0 ** -24, 1e-4)])
def test_columns_with_scale_negatives_match_oracle(precision, eps, floor):
    cuda()
    from test_gpu_columns import add_all, assert_within_envelope, lobster_cols, oracle_columns, perturbed
    bgc = obgc.LOBSTER(None, carbonate_system=obgc.CarbonateSystem(), scale_negatives=True)
    cols = lobster_cols(n=16, seed=21)
    eng = obgc.ColumnEngine(bgc, precision=precision, max_columns=16, arena_cells=16 * 520)
    slots = add_all(eng, cols)
    while any(eng.remaining(s) for s in slots):
        eng.advance(64)
    got = [eng.read(s) for s in slots]
    ref = oracle_columns(bgc, cols, eng.tracers, negatives=O.NEG_SCALE)
    pert = oracle_columns(bgc, perturbed(cols, eps), eng.tracers, negatives=O.NEG_SCALE)
    assert_within_envelope(got, ref, pert, floor)
    nh4 = eng.tracers.index("NH₄")
    assert min(np.min(g[nh4]) for g in got) >= 0.0
