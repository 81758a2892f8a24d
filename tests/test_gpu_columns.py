"""GPU parity of the packed uneven-column engine against the oracle's column runner (FP64 and FP32),
and its batching properties: a column's result does not depend on the columns it shares a pack or
a launch with, on how its steps are split over launches, or on graph replay."""
import numpy as np
import pytest

import obgc
import oracle as O
from gpuhelp import cuda, rel_err

pytestmark = pytest.mark.gpu


def oracle_columns(bgc, cols, names, negatives=O.NEG_NONE, gas=None):
    """Run the columns through the oracle; returns a list of [n_tracers, Nz] arrays."""
    nt = len(names)
    so, ko, states, kaps, specs = [], [], [], [], []
    s_off = k_off = 0
    for c in cols:
        Nz = c["init"].shape[1]
        so.append(s_off)
        ko.append(k_off)
        states.append(c["init"].ravel())
        kaps.append(c["kappa"])
        s_off += nt * Nz
        k_off += Nz + 1
        specs.append(O.Column(Nz, c["nsteps"], c["dz"], c["surface_PAR"], c.get("mu0", 0.0), c["dt"],
                              c.get("pulse_step", -1), c.get("pulse_k", -1), c.get("pulse_amount", 0.0),
                              c.get("T", 15.0), c.get("S", 35.0)))
    state = np.ascontiguousarray(np.concatenate(states))
    kappa = np.ascontiguousarray(np.concatenate(kaps))
    O.columns_run(bgc.params, bgc.light_attenuation.params if bgc.light_attenuation else obgc._abi.default_twoband(),
                  specs, names, state, kappa, so, ko, 0.0, 0, negatives=negatives,
                  invalid_fill_value=getattr(bgc, "invalid_fill_value", float("nan")), gas=gas)
    return [state[so[q]:so[q] + nt * c["init"].shape[1]].reshape(nt, -1) for q, c in enumerate(cols)]


def add_all(eng, cols):
    return [eng.add(c["init"], c["kappa"], c["dz"], c["dt"], c["nsteps"], surface_PAR=c["surface_PAR"],
                    mu0=c.get("mu0", 0.0), pulse_step=c.get("pulse_step", -1), pulse_k=c.get("pulse_k", -1),
                    pulse_amount=c.get("pulse_amount", 0.0), T=c.get("T", 15.0), S=c.get("S", 35.0)) for c in cols]


def npzd_cols(n=48, nsteps=60, seed=3):
    return obgc.npzd_column_ensemble(n, seed=seed, levels=(16, 256), nsteps=nsteps)


def lobster_cols(n=24, seed=5, days=(0.2, 1.5)):
    rng = np.random.default_rng(seed)
    return [obgc.lobster_column_request(rng, days=days) for _ in range(n)]


def lobster_bgc():
    return obgc.LOBSTER(None, carbonate_system=obgc.CarbonateSystem())


def perturbed(cols, eps, seed=0):
    """The columns with the initial state perturbed by eps-relative noise and dt scaled by 1 + eps, so
    that every RK3 increment moves by eps relative: the size of the error that rounding the
    tendencies in the engine's compute precision injects at every stage."""
    rng = np.random.default_rng(seed)
    return [dict(c, init=c["init"] * (1 + eps * rng.standard_normal(c["init"].shape)), dt=c["dt"] * (1 + eps))
            for c in cols]


def assert_within_envelope(got, ref, pert, floor, factor=10.0):
    """The stated tolerance of the column path: per column and tracer,
    max|got - ref| <= factor * max|pert - ref| + floor * max|ref|, where pert is the oracle's own
    result from inputs and increments perturbed by one unit roundoff of the engine's compute
    precision (perturbed()).  Near-depleted
    cells (NH4 oscillating about zero under strong light) amplify any rounding difference by up to
    1e6 in the reference algorithm itself, so a fixed relative bound would test the conditioning of
    the model, not the engine."""
    worst = 0.0
    for g, r, p in zip(got, ref, pert):
        for q in range(r.shape[0]):
            allowed = factor * np.max(np.abs(p[q] - r[q])) + floor * np.max(np.abs(r[q]))
            err = np.max(np.abs(g[q] - r[q]))
            assert err <= allowed, (q, err, allowed)
            worst = max(worst, err / max(np.max(np.abs(r[q])), 1e-300))
    return worst


def max_err(got, ref):
    return max(max(rel_err(g[q], r[q], floor_frac=1e-3) for q in range(g.shape[0])) for g, r in zip(got, ref))


@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("f32", 2e-4), ("mixed", 2e-4)])
def test_npzd_columns_match_oracle(precision, tol):
    cuda()
    bgc = obgc.NPZD(None)
    cols = npzd_cols()
    eng = obgc.ColumnEngine(bgc, precision=precision, max_columns=64, arena_cells=64 * 300)
    slots = add_all(eng, cols)
    eng.advance(25)
    eng.advance(100)
    assert all(eng.remaining(s) == 0 for s in slots)
    got = [eng.read(s) for s in slots]
    ref = oracle_columns(bgc, cols, eng.tracers)
    err = max_err(got, ref)
    assert err < tol, err
    assert max(np.max(np.abs(r - c["init"])) for r, c in zip(ref, cols)) > 1e-3   # the columns did evolve


# floor: FP32 tendencies round each source and sink term, and where they nearly cancel (NH4 uptake
# against remineralisation) the per-step error is eps * sum|terms| * dt, above the envelope's
# eps * |net| * dt: up to ~5e-5 of the column maximum after a few hundred steps, in FP32 and in
# mixed precision alike (mixed keeps the state in FP64, the tendencies are FP32).  FP32 state also
# loses the part of each increment below half a unit in the last place of DIC and Alk (about 2000,
# so 6e-5 absolute), which mixed precision keeps.
@pytest.mark.parametrize("precision,eps,floor", [("f64", 2.0 ** -53, 1e-12), ("f32", 2.0 ** -24, 1e-4),
                                                 ("mixed", 2.0 ** -24, 1e-4)])
def test_lobster_columns_with_pulses_match_oracle(precision, eps, floor):
    cuda()
    bgc = lobster_bgc()
    cols = lobster_cols()
    eng = obgc.ColumnEngine(bgc, precision=precision, max_columns=32, arena_cells=32 * 520)
    slots = add_all(eng, cols)
    while any(eng.remaining(s) for s in slots):
        eng.advance(37)
    got = [eng.read(s) for s in slots]
    ref = oracle_columns(bgc, cols, eng.tracers)
    pert = oracle_columns(bgc, perturbed(cols, eps), eng.tracers)
    assert_within_envelope(got, ref, pert, floor)


@pytest.mark.parametrize("precision,eps,floor", [("f64", 2.0 ** -53, 1e-12), ("mixed", 2.0 ** -24, 1e-4),
                                                 ("f32", 2.0 ** -24, 1e-4)])
def test_lobster_columns_with_co2_exchange_match_oracle(precision, eps, floor):
    # examples/column.jl:54-64: the CO2 gas exchange on every column's DIC, each column with its own
    # surface T and S, a wind of 8 m/s and the air's 413 ppm; the alkalinity pulses then drive uptake
    cuda()
    bgc = lobster_bgc()
    cols = lobster_cols()   # the columns of the test above (their NH4 is within the envelope in mixed precision)
    co2 = obgc.CarbonDioxideGasExchangeBoundaryCondition(wind_speed=8.0)
    eng = obgc.ColumnEngine(bgc, precision=precision, max_columns=32, arena_cells=32 * 520, co2_exchange=co2)
    slots = add_all(eng, cols)
    while any(eng.remaining(s) for s in slots):
        eng.advance(37)
    got = [eng.read(s) for s in slots]
    ref = oracle_columns(bgc, cols, eng.tracers, gas=co2.params)
    pert = oracle_columns(bgc, perturbed(cols, eps), eng.tracers, gas=co2.params)
    assert_within_envelope(got, ref, pert, floor)
    # the condition moved the surface DIC (and nothing the pulses alone would)
    plain = oracle_columns(bgc, cols, eng.tracers)
    q = eng.tracers.index("DIC")
    assert max(abs(r[q, -1] - p[q, -1]) for r, p in zip(ref, plain)) > 1e-2


def test_result_is_the_same_alone_and_in_the_mix():
    """Continuous batching must not change a column's result: the same column run alone, and run
    while other columns join and leave the engine at other steps, is bit-for-bit the same."""
    cuda()
    bgc = lobster_bgc()
    cols = lobster_cols(n=12, seed=11, days=(0.3, 1.0))
    probe = cols[0]
    alone = obgc.ColumnEngine(bgc, precision="f32", max_columns=4, arena_cells=2048)
    s = add_all(alone, [probe])[0]
    while alone.remaining(s):
        alone.advance(50)
    ref = alone.read(s)

    mixed = obgc.ColumnEngine(bgc, precision="f32", max_columns=32, arena_cells=32 * 520)
    others = add_all(mixed, cols[1:6])
    mixed.advance(7)                       # the others start earlier
    sp = add_all(mixed, [probe])[0]
    pending = list(cols[6:])
    while mixed.remaining(sp):
        mixed.advance(13)
        for o in list(others):
            if mixed.remaining(o) == 0:
                mixed.remove(o)
                others.remove(o)
        if pending:                        # new requests arrive while the probe is in flight
            others += add_all(mixed, [pending.pop()])
    got = mixed.read(sp)
    assert np.array_equal(got, ref)


def test_graph_run_equals_launch_by_launch():
    cuda()
    bgc = obgc.NPZD(None)
    cols = npzd_cols(n=40, nsteps=30, seed=9)
    a = obgc.ColumnEngine(bgc, precision="f32", max_columns=64, arena_cells=64 * 300)
    b = obgc.ColumnEngine(bgc, precision="f32", max_columns=64, arena_cells=64 * 300)
    sa, sb = add_all(a, cols), add_all(b, cols)
    for _ in range(30):
        a.advance(1)
    b.run(20, steps_per_launch=1, graph=True)     # capture + replay
    b.run(10, steps_per_launch=4, graph=True)
    for x, y in zip(sa, sb):
        assert b.remaining(y) == 0
        assert np.array_equal(a.read(x), b.read(y))


def test_arena_budget_and_reuse():
    cuda()
    bgc = obgc.NPZD(None)
    eng = obgc.ColumnEngine(bgc, precision="f32", max_columns=8, arena_cells=300)
    init = lambda Nz: np.tile(np.array([[5.0], [0.03], [0.03], [12.0], [0.0]]), (1, Nz))   # noqa: E731
    k = lambda Nz: np.full(Nz + 1, 1e-3)                                                 # noqa: E731
    s1 = eng.add(init(99), k(99), 2.0, 600.0, 2)     # 100 cells
    s2 = eng.add(init(99), k(99), 2.0, 600.0, 2)     # 200
    s3 = eng.add(init(99), k(99), 2.0, 600.0, 2)     # 300: full
    with pytest.raises(obgc._abi.ObgcError) as ei:
        eng.add(init(10), k(10), 2.0, 600.0, 2)
    assert ei.value.status == 8                      # OBGC_ERR_BUSY
    eng.remove(s1)
    eng.remove(s2)                                   # coalesces into 200 free cells
    s4 = eng.add(init(180), k(180), 2.0, 600.0, 2)
    eng.advance(5)
    assert eng.remaining(s3) == 0 and eng.remaining(s4) == 0
    with pytest.raises(obgc._abi.ObgcError):
        eng.remaining(7)                             # never used
    with pytest.raises(obgc._abi.ObgcError):
        eng.remove(7)


def test_autotune_restores_state():
    cuda()
    bgc = obgc.NPZD(None)
    cols = npzd_cols(n=40, nsteps=12, seed=4)
    a = obgc.ColumnEngine(bgc, precision="f32", max_columns=64, arena_cells=64 * 300)
    b = obgc.ColumnEngine(bgc, precision="f32", max_columns=64, arena_cells=64 * 300)
    sa, sb = add_all(a, cols), add_all(b, cols)
    threads, cells = b.autotune(steps=3)
    assert threads % 32 == 0 and cells >= 512
    a.advance(12)
    b.advance(12)
    for x, y in zip(sa, sb):
        assert np.array_equal(a.read(x), b.read(y))
