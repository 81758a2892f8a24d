"""The oracle's NutrientsPlanktonDetritus functors and BoxModel RK3.

Mirrors test/test_NutrientsPlanktonDetritus.jl: the 72 component combinations, zero stays zero,
and nitrogen / carbon conservation over 100 steps of 1 s with random initial values
(test_NutrientsPlanktonDetritus.jl:27-139), plus the LOBSTER / NPZD tracer lists of the
constructor doctests (constructors.jl:56-57, 168-169).
"""
import itertools

import numpy as np
import pytest

import oracle as O
from obgc import _abi as A

NUTS = (A.NUT_NITRATE_AMMONIA, A.NUT_NITRATE_AMMONIA_IRON, A.NUT_NUTRIENT)
DETS = (A.DET_TWO_PARTICLE, A.DET_VARIABLE_REDFIELD, A.DET_SINGLE)


def configs():
    for sinking, det, oxy, carb, nut in itertools.product((False, True), DETS, (0, 1), (0, 1), NUTS):
        p = O.preset("LOBSTER")
        p.nutrients, p.detritus, p.oxygen, p.carbonate_system = nut, det, oxy, carb
        if not sinking:
            p.small_particle_sinking_speed = p.large_particle_sinking_speed = 0.0
            p.detritus_sinking_speed = 0.0
        else:
            p.detritus_sinking_speed = 0.1213 / 86400
        yield sinking, p


def initial_values(p, rng):
    v = {"P": rng.random(), "Z": rng.random()}
    if p.nutrients == A.NUT_NITRATE_AMMONIA:
        v.update(NO3=10 * rng.random(), NH4=rng.random())
    elif p.nutrients == A.NUT_NITRATE_AMMONIA_IRON:
        v.update(NO3=10 * rng.random(), NH4=rng.random(), Fe=1e-3 * rng.random())
    else:
        v.update(N=10 * rng.random())
    if p.carbonate_system:
        v.update(DIC=2000 * rng.random(), Alk=2000 * rng.random())
    if p.oxygen:
        v.update(O2=300 * rng.random())
    if p.detritus == A.DET_VARIABLE_REDFIELD:
        a, b, c = rng.random(), rng.random(), rng.random()
        v.update(sPON=a, bPON=b, DON=c, sPOC=6.56 * a, bPOC=6.56 * b, DOC=6.56 * c)
    elif p.detritus == A.DET_TWO_PARTICLE:
        v.update(sPOM=rng.random(), bPOM=rng.random(), DOM=rng.random())
    else:
        v.update(D=rng.random())
    return v


def nitrogen(p, v):
    names = ["P", "Z"] + (["NO3", "NH4"] if p.nutrients != A.NUT_NUTRIENT else ["N"])
    names += {A.DET_VARIABLE_REDFIELD: ["sPON", "bPON", "DON"], A.DET_TWO_PARTICLE: ["sPOM", "bPOM", "DOM"]}.get(p.detritus, ["D"])
    return sum(v[A.NAME_INDEX[n]] for n in names)


def carbon(p, v):
    R, rho = p.redfield_ratio, p.carbon_calcite_ratio
    tot = v[A.OBGC_P] * (1 + rho) * R + v[A.OBGC_Z] * R + v[A.OBGC_DIC]
    if p.detritus == A.DET_VARIABLE_REDFIELD:
        tot += v[A.OBGC_SPOC] + v[A.OBGC_BPOC] + v[A.OBGC_DOC]
    elif p.detritus == A.DET_TWO_PARTICLE:
        tot += R * (v[A.OBGC_SPOM] + v[A.OBGC_BPOM] + v[A.OBGC_DOM])
    else:
        tot += R * v[A.OBGC_D]
    return tot


ALL = list(configs())


def test_72_configurations():
    assert len(ALL) == 72


@pytest.mark.parametrize("idx", range(72))
def test_zero_stays_zero(idx):
    _, p = ALL[idx]
    v = O.box_run(p, {}, 1.0, 1, PAR_const=100.0)
    assert np.all(v == 0)


def test_conservation():
    rng = np.random.default_rng(42)
    for sinking, p in ALL:
        vals = initial_values(p, rng)
        if sinking:
            continue
        v0 = O.box_run(p, vals, 1.0, 0, PAR_const=100.0)
        v1 = O.box_run(p, vals, 1.0, 100, PAR_const=100.0)
        assert nitrogen(p, v1) == pytest.approx(nitrogen(p, v0), rel=1.5e-8)
        if p.carbonate_system:
            assert carbon(p, v1) == pytest.approx(carbon(p, v0), rel=1.5e-8)
        assert not np.allclose(v0, v1)   # something happened


def test_tendencies_conserve_instantaneously():
    # the sum of N tendencies is zero to rounding for every configuration (no sinking involved)
    rng = np.random.default_rng(7)
    for _, p in ALL:
        vals = initial_values(p, rng)
        names = O.required_tracers(p)
        G = {n: O.tendency(p, n, vals, 37.0) for n in names}
        g = np.zeros(A.NUM_NAMED)
        for n, x in G.items():
            g[n] = x
        scale = max(abs(x) for x in G.values())
        assert abs(nitrogen(p, g)) <= 1e-12 * scale
        if p.carbonate_system:
            assert abs(carbon(p, g)) <= 1e-12 * scale * 10


def test_constructor_tracer_lists():
    lob = [A.ASCII_NAMES[i] for i in O.required_tracers(O.preset("LOBSTER"))]
    npzd = [A.ASCII_NAMES[i] for i in O.required_tracers(O.preset("NPZD"))]
    assert lob == ["NO3", "NH4", "P", "Z", "sPOM", "bPOM", "DOM"]
    assert npzd == ["N", "P", "Z", "T", "D"]


def test_npzd_box_model_runs():
    # examples/box.jl / benchmark/box_model.jl: NPZD, N=10, P=0.1, Z=0.01, dt = 20 min, 1000 steps
    p = O.preset("NPZD")
    v = O.box_run(p, {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 10.0}, 1200.0, 1000, PAR_const=20.0)
    assert np.all(np.isfinite(v))
    assert nitrogen(p, v) == pytest.approx(10.11, rel=1e-9)
