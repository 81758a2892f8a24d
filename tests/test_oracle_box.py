"""Oracle (CPU) of BoxModel(; forcing, prescribed_tracers) (src/BoxModel/boxmodel.jl:65-106,
timesteppers.jl:37-63): the forms the GPU BoxModel kernel is checked against."""
import math

import numpy as np
import pytest

import obgc
import oracle as O
from obgc import _abi as A


def npzd():
    return obgc.NPZD(obgc.BoxModelGrid(), light_attenuation=obgc.PrescribedPhotosyntheticallyActiveRadiation(40.0))


def test_constant_forcing_of_a_tracer_without_tendency_integrates_exactly():
    # NPZD carries T with no tendency: a constant rate r raises it by r dt per step (the RK3 stage
    # weights of a step sum to one)
    bgc = npzd()
    dt, nsteps, r = 600.0, 50, 1e-5
    v = O.box_run_drivers(bgc.params, {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 12.0}, dt, nsteps, PAR_const=40.0,
                          forcing={"T": np.full(3 * nsteps, r)})
    assert v[A.NAME_INDEX["T"]] == pytest.approx(12.0 + r * dt * nsteps, rel=1e-14)


def test_prescribed_tracer_holds_its_value_at_the_end_and_drives_growth():
    bgc = npzd()
    dt, nsteps = 600.0, 40
    f = lambda t: 5.0 + t / 86400.0          # noqa: E731
    times = [dt * (s + c) for s in range(nsteps + 1) for c in (0, 8 / 15, 2 / 3)][:3 * nsteps + 1]
    v = O.box_run_drivers(bgc.params, {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 0.0}, dt, nsteps, PAR_const=40.0,
                          prescribed={"T": [f(t) for t in times]})
    assert v[A.NAME_INDEX["T"]] == f(dt * nsteps)
    # a constant prescription equals the plain run started at that temperature
    c = O.box_run_drivers(bgc.params, {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 0.0}, dt, nsteps, PAR_const=40.0,
                          prescribed={"T": np.full(3 * nsteps + 1, 14.0)})
    plain = O.box_run(bgc.params, {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 14.0}, dt, nsteps, PAR_const=40.0)
    np.testing.assert_array_equal(c, plain)
    # warmer water grows faster (Q10): the rising temperature left more P than a cold constant one
    cold = O.box_run(bgc.params, {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 5.0}, dt, nsteps, PAR_const=40.0)
    assert v[A.NAME_INDEX["P"]] > cold[A.NAME_INDEX["P"]]


def test_no_drivers_is_the_plain_box_run():
    bgc = npzd()
    init = {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 12.0}
    par = np.array([40.0 * (1 + math.sin(q)) for q in range(3 * 30)])
    np.testing.assert_array_equal(O.box_run_drivers(bgc.params, init, 900.0, 30, PAR_stages=par),
                                  O.box_run(bgc.params, init, 900.0, 30, PAR_stages=par))


def test_box_model_rejects_unknown_driver_names():
    bgc = npzd()
    with pytest.raises(ValueError):
        obgc.BoxModel(bgc, forcing={"NO3": 1.0})
