"""The oracle's SimpleMultiGSediment (nitrogen-only form, src/Models/Sediments/simple_multi_G.jl)
coupled to a LOBSTER + Oxygen water column: nitrogen conserved between the water and the sediment,
the coupled tendencies return exactly the remineralised nitrogen, a zero sediment with nothing
sinking couples nothing, and the library's host parameters are the reference's defaults."""
import ctypes as C

import numpy as np

import obgc
import oracle as O
from obgc import _abi as A

NAMES = ["NO3", "NH4", "P", "Z", "sPOM", "bPOM", "DOM", "O2"]


def lobster_o2(shape=(4, 4, 12)):
    g = obgc.RectilinearGrid(shape, (400.0, 400.0, 120.0))
    bgc = obgc.LOBSTER(g, oxygen=obgc.Oxygen())
    bgc.params.open_bottom = 1
    rng = np.random.default_rng(2)
    init = dict(NO3=10.0, NH4=0.5, P=0.5, Z=0.1, sPOM=1.0, bPOM=1.0, DOM=0.1, O2=250.0)
    st = np.ascontiguousarray(np.stack([np.full(g.shape, init[n]) * np.exp(0.1 * rng.standard_normal(g.shape))
                                        for n in NAMES]))
    return g, bgc, st


def default_params():
    p = A.MultiGParams()
    assert A.load().obgc_multig_default_params(C.byref(p)) == 0
    return p


def test_defaults_are_the_references():
    p = default_params()
    assert abs(p.fast_decay_rate - 2 / 86400) < 1e-20 and abs(p.slow_decay_rate - 0.2 / 86400) < 1e-20
    assert (p.fast_fraction, p.slow_fraction, p.refactory_fraction) == (0.74, 0.26, 0.1)
    assert (p.anoxia_half_saturation, p.sinking_redfield) == (1.0, 6.56)
    assert list(p.nitrate_oxidation) == [-1.9785, 0.2261, -0.0615, -0.0289, -0.36109, -0.0232]
    assert list(p.denitrification) == [-3.0790, 1.7509, 0.0593, -0.1923, 0.0604, 0.0662]
    assert list(p.anoxic) == [-3.9476, 2.6269, -0.2426, -1.3349, 0.1826, -0.0143]


def nitrogen_drift(dt, nsteps):
    """Relative change of water + sediment nitrogen over nsteps, and the final state and sediment."""
    g, bgc, st = lobster_o2()
    m = O.model3d(bgc.params, g.c_grid(), NAMES)
    sed = O.attach_multig(m, default_params(), NAMES, ("sPOM", "bPOM"), g)
    dV, dA = g.Lx * g.Ly * g.Lz / g.N, g.Lx * g.Ly / (g.Nx * g.Ny)
    NN = g.Nx * g.Ny
    nitrogen = [NAMES.index(n) for n in ("NO3", "NH4", "P", "Z", "sPOM", "bPOM", "DOM")]

    def total(s):
        return sum(s[q].sum() for q in nitrogen) * dV + sed[:3 * NN].sum() * dA
    n0 = total(st)
    O.step3d(m, st, t=0.0, dt=dt, nsteps=nsteps)
    return (total(st) - n0) / n0, st, sed, NN, bgc, g


def test_nitrogen_is_conserved_between_water_and_sediment():
    """The water loses through the bottom face what the sediment gains, and gets back what it
    remineralises (F_NO3 + F_NH4 = the remineralisation rate).  In discrete time the coupling is
    lagged as the reference's is (the sediment steps after each water stage on the fluxes tracked
    then), so the budget closes to first order in dt: the imbalance halves with dt."""
    d600, st, sed, NN, bgc, g = nitrogen_drift(600.0, 40)
    d300, *_ = nitrogen_drift(300.0, 80)
    assert np.all(sed[:3 * NN] > 0)             # deposited
    assert np.all(sed[3 * NN:] == 1.0)          # the sediment's clock has started
    assert abs(d600) < 2e-5
    assert 1.8 < d600 / d300 < 2.3
    # the sediment returns nitrogen: the bottom cells' NH4 exceeds a run without a sediment
    m0 = O.model3d(bgc.params, g.c_grid(), NAMES)
    _, _, st0 = lobster_o2()
    O.step3d(m0, st0, t=0.0, dt=600.0, nsteps=40)
    assert np.all(st[NAMES.index("NH4")][0] > st0[NAMES.index("NH4")][0])


def test_empty_sediment_with_nothing_sinking_couples_nothing():
    g, bgc, st = lobster_o2()
    st[NAMES.index("sPOM")] = 0.0
    st[NAMES.index("bPOM")] = 0.0
    m = O.model3d(bgc.params, g.c_grid(), NAMES)
    sed = O.attach_multig(m, default_params(), NAMES, ("sPOM", "bPOM"), g)
    ref = st.copy()
    m0 = O.model3d(bgc.params, g.c_grid(), NAMES)
    O.step3d(m, st, t=0.0, dt=600.0, nsteps=1)
    O.step3d(m0, ref, t=0.0, dt=600.0, nsteps=1)
    NN = g.Nx * g.Ny
    # the first stages deposit the detritus the functors make; before any deposition nothing returns
    assert np.all(np.isfinite(st)) and np.all(sed[:3 * NN] >= 0)
    assert np.max(np.abs(st - ref) / np.abs(ref).max(axis=(1, 2, 3), keepdims=True)) < 1e-6
