"""Oracle (CPU) properties of CarbonateSystem(N) replicates and tracer forcing in the 3-D step, and
the library's host-side naming of the replicated tracers.

carbonate_system.jl:41-83: CarbonateSystem(N) carries DIC1..DICN and Alk1..AlkN, each replicate
evaluating the DIC / Alk functor; the replicates therefore differ only through their boundary
conditions and forcing (examples/oae_experiment.jl)."""
import numpy as np
import pytest

import obgc
import oracle as O
from obgc import _abi as A


def small_case(seed=3, shape=(12, 8, 6)):
    g = obgc.RectilinearGrid(shape, (500.0, 400.0, 15.0))
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(2))
    rng = np.random.default_rng(seed)
    names = ["NO3", "NH4", "P", "Z", "sPOM", "bPOM", "DOM", "DIC", None, "Alk", None, "T", "S"]
    base = dict(NO3=10.0, NH4=0.1, P=0.5, Z=0.2, sPOM=0.05, bPOM=0.02, DOM=0.1, DIC=2000.0, Alk=2300.0, T=15.0, S=35.0)
    state = np.zeros((len(names),) + g.shape)
    for q, n in enumerate(names):
        key = n if n is not None else ("DIC" if q == 8 else "Alk")
        state[q] = base[key] * (1 + 0.05 * rng.standard_normal(g.shape))
    state[8], state[10] = state[7], state[9]     # the replicates start equal
    u = rng.normal(0, 0.01, g.shape).ravel().copy()
    v = rng.normal(0, 0.01, g.shape).ravel().copy()
    return g, bgc, names, state, u, v


def test_required_tracers_of_replicated_carbonate_system():
    g = obgc.RectilinearGrid((4, 4, 4), (1.0, 1.0, 1.0))
    one = obgc.required_biogeochemical_tracers(obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem()))
    three = obgc.required_biogeochemical_tracers(obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(3)))
    assert one[7:] == ("DIC", "Alk")
    assert three[:7] == one[:7]
    assert three[7:] == ("DIC1", "DIC2", "DIC3", "Alk1", "Alk2", "Alk3")
    with pytest.raises(ValueError):
        obgc.CarbonateSystem(0)


def test_replicate_evaluates_the_carbonate_functor():
    g = obgc.RectilinearGrid((4, 4, 4), (1.0, 1.0, 1.0))
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(2))
    vals = dict(NO3=10.0, NH4=0.3, P=0.6, Z=0.3, sPOM=0.1, bPOM=0.05, DOM=0.2, DIC1=2000.0, Alk1=2300.0)
    for rep, base in (("DIC2", "DIC1"), ("Alk2", "Alk1")):
        assert obgc.eval_point(bgc, rep, vals, 40.0) == obgc.eval_point(bgc, base, vals, 40.0) != 0.0


def test_replicates_started_equal_stay_equal_in_the_oracle():
    g, bgc, names, state, u, v = small_case()
    m = O.model3d(bgc.params, g.c_grid(), names, tendency_of={8: "DIC", 10: "Alk"})
    O.step3d(m, state, u=u, v=v, t=0.0, dt=300.0, nsteps=3)
    assert np.array_equal(state[8], state[7]) and np.array_equal(state[10], state[9])
    # and a passive slot without a source only moves with the flow
    g2, bgc2, names2, s2, u2, v2 = small_case()
    m2 = O.model3d(bgc2.params, g2.c_grid(), names2, tendency_of={8: "DIC"})
    O.step3d(m2, s2, u=u2, v=v2, t=0.0, dt=300.0, nsteps=3)
    assert np.array_equal(s2[8], state[8])
    assert s2[10].sum() == pytest.approx(small_case()[3][10].sum(), rel=1e-13)


def test_oracle_forcing_window_releases_its_integral():
    g, bgc, names, state, u, v = small_case()
    rate = np.zeros(g.shape)
    rate[-1, 2:5, 3:8] = 0.03
    before = state.copy()
    m = O.model3d(bgc.params, g.c_grid(), names, tendency_of={8: "DIC", 10: "Alk"}, forcing={10: (rate, 300.0, 900.0)})
    O.step3d(m, state, u=u, v=v, t=0.0, dt=300.0, nsteps=4)
    released = (state[10] - state[9]).sum() - (before[10] - before[9]).sum()
    assert released == pytest.approx(rate.sum() * 2 * 300.0, rel=1e-10)
    # a window that holds only the last stage of a step (t + 2/3 dt = 200 s) adds its RK3 weight 3/4
    g, bgc, names, state, u, v = small_case()
    before = state.copy()
    m = O.model3d(bgc.params, g.c_grid(), names, tendency_of={8: "DIC", 10: "Alk"}, forcing={10: (rate, 190.0, 210.0)})
    O.step3d(m, state, u=u, v=v, t=0.0, dt=300.0, nsteps=1)
    released = (state[10] - state[9]).sum() - (before[10] - before[9]).sum()
    assert released == pytest.approx(rate.sum() * 0.75 * 300.0, rel=1e-10)


def test_model_desc_carries_passive_sources():
    d = A.ModelDesc()
    assert len(d.passive_tendency_of) == A.MAX_PASSIVE
    assert A.PASSIVE(0) == A.NUM_NAMED
