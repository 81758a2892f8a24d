"""The oracle's conditioning probe (or_model3d.stage_rounding) and its stage-level step on small
cases: the probe is off by default, it perturbs by the stated relative size, the sensitivity it
exposes in the 3-D step comes from advection, not from the BGC functors, and three stages of
or_stage3d are one step of or_step3d."""
import numpy as np

import conditioning as K


def test_zero_rounding_is_the_plain_step():
    c = K.LobsterCase((16, 16, 8))
    a = c.oracle_run(20)
    b = c.oracle_run(20, stage_rounding=0.0, seed=7)
    assert np.array_equal(a, b)


def test_rounding_of_one_stage_has_the_stated_size():
    c = K.LobsterCase((8, 8, 4))
    import oracle as O
    m0 = O.model3d(c.bgc.params, c.grid.c_grid(), K.NAMES)
    m1 = O.model3d(c.bgc.params, c.grid.c_grid(), K.NAMES)
    m1.stage_rounding, m1.rounding_seed = 1e-6, 3
    a, b = c.state0.copy(), c.state0.copy()
    O.step3d(m0, a, u=c.u, v=c.v, t=0.0, dt=K.DT, nsteps=1)
    O.step3d(m1, b, u=c.u, v=c.v, t=0.0, dt=K.DT, nsteps=1)
    r = np.abs(b - a) / np.abs(a)
    # three stages, each one factor (1 +/- 1e-6) on every value
    assert 0.5e-6 < np.median(r) < 3.5e-6
    assert r.max() < 1e-5     # neighbours' perturbations also enter through the fluxes


def test_bgc_alone_is_well_conditioned():
    """With advection off the functors and light carry an FP64 rounding per stage at its own
    size: the sensitivity of the 3-D step lies in the WENO5 advection."""
    c = K.LobsterCase((8, 8, 8))
    import oracle as O
    runs = []
    for r in (0.0, K.U64):
        m = O.model3d(c.bgc.params, c.grid.c_grid(), K.NAMES, advection=0)
        m.stage_rounding, m.rounding_seed = r, 1
        s = c.state0.copy()
        O.step3d(m, s, u=c.u, v=c.v, t=0.0, dt=K.DT, nsteps=300)
        runs.append(s)
    stmt = K.error_statement(runs[1], runs[0])
    assert max(e["max_rel"] for e in stmt.values()) < 1e-12


def test_three_stages_are_one_step():
    c = K.LobsterCase((16, 16, 8))
    import oracle as O
    a = c.oracle_run(3)
    m = O.model3d(c.bgc.params, c.grid.c_grid(), K.NAMES)
    s = c.state0.copy()
    G, Gm = np.zeros_like(s), np.zeros_like(s)
    for n in range(3):
        for st in range(3):
            O.stage3d(m, s, G, Gm, u=c.u, v=c.v, t=n * K.DT, dt=K.DT, stage=st)
            G, Gm = Gm, G
    assert np.array_equal(a, s)
