"""Negative-tracer modifiers in the oracle, pinned to the reference's own known answers
(test/test_utils.jl:7-40) and to conserved_tracers (coupling_utils.jl:1-52)."""
import math

import numpy as np
import pytest

import obgc
import oracle as O


def one_cell(bgc, values, negatives, zero_exclude=()):
    g = obgc.RectilinearGrid((1, 1, 1), (1.0, 1.0, 1.0))
    names = obgc.required_biogeochemical_tracers(bgc)
    m = O.model3d(bgc.params, g.c_grid(), names, negatives=negatives, zero_exclude=zero_exclude)
    state = np.array([[values.get(n, 0.0)] for n in names], dtype=np.float64)
    O.step3d(m, state, t=0.0, dt=1e-10, nsteps=1)
    return {n: state[q, 0] for q, n in enumerate(names)}


def test_scale_negative_tracers_known_answer():
    # test_negative_scaling: NPZD(grid; scale_negatives = true), set!(N = 2, P = -1), one step of 1e-10 s
    out = one_cell(obgc.NPZD(None), {"N": 2.0, "P": -1.0}, O.NEG_SCALE)
    assert out["N"] == pytest.approx(1.0, rel=1e-8)
    assert out["P"] == pytest.approx(0.0, abs=1e-8)


def test_zero_negative_tracers_known_answer():
    # test_negative_zeroing: ZeroNegativeTracers(; exclude = (:Z,)), set!(N = 2, P = -1, Z = -1)
    out = one_cell(obgc.NPZD(None), {"N": 2.0, "P": -1.0, "Z": -1.0}, O.NEG_ZERO, zero_exclude=("Z",))
    assert out["N"] == pytest.approx(2.0, rel=1e-8)
    assert out["P"] == pytest.approx(0.0, abs=1e-8)
    assert out["Z"] == pytest.approx(-1.0, rel=1e-6)


@pytest.mark.parametrize("make", [
    lambda: obgc.NPZD(None),
    lambda: obgc.LOBSTER(None),
    lambda: obgc.LOBSTER(None, carbonate_system=obgc.CarbonateSystem()),
    lambda: obgc.LOBSTER(None, detritus=obgc.VariableRedfieldDetritus(), carbonate_system=obgc.CarbonateSystem()),
])
def test_conserved_groups_match_conserved_tracers(make):
    bgc = make()
    names = obgc.required_biogeochemical_tracers(bgc)
    groups = O.conserved_groups(bgc.params, names)
    expect = obgc.conserved_tracers(bgc)
    if not bgc.params.carbonate_system:
        expect = (expect,)
    assert len(groups) == len(expect)
    for (slots, factors), e in zip(groups, expect):
        tr, sf = (e, (1.0,) * len(e)) if isinstance(e, tuple) else (e["tracers"], e["scalefactors"])
        assert [names[q] for q in slots] == [obgc._abi.ASCII_NAMES[obgc._abi.NAME_INDEX[t]] for t in tr]
        assert factors == pytest.approx(list(sf), rel=0, abs=0)


def test_scale_cell_rules():
    bgc = obgc.LOBSTER(None, carbonate_system=obgc.CarbonateSystem())
    names = obgc.required_biogeochemical_tracers(bgc)
    groups = O.conserved_groups(bgc.params, names)
    gn, gs, gf = O.group_arrays(groups)
    P = O.C.POINTER
    v = np.array([1.0, 0.5, -0.1, 0.2, 0.3, -0.05, 0.1, 2000.0, 2300.0])
    ref = v.copy()
    # nitrogen group first, then carbon, each with the previous group's result
    for sl, fa in groups:
        x = ref[sl] * np.array(fa)
        t, p = x.sum(), x[ref[sl] > 0].sum()
        ref[sl] = np.where(ref[sl] > 0, ref[sl] * t / p, 0.0)
    O.lib().or_scale_cell(v.ctypes.data_as(P(O.C.c_double)), 1, len(groups), gn.ctypes.data_as(P(O.C.c_int32)),
                          gs.ctypes.data_as(P(O.C.c_int32)), gf.ctypes.data_as(P(O.C.c_double)), math.nan)
    np.testing.assert_allclose(v, ref, rtol=1e-15)
    assert v[names.index("Alk")] == 2300.0
    # a negative total fills with invalid_fill_value (NaN by default)
    w = np.array([-1.0, 0.0, 0.5, 0.1, 0.0, 0.0, 0.0, 2000.0, 2300.0])
    O.lib().or_scale_cell(w.ctypes.data_as(P(O.C.c_double)), 1, 1, gn.ctypes.data_as(P(O.C.c_int32)),
                          gs.ctypes.data_as(P(O.C.c_int32)), gf.ctypes.data_as(P(O.C.c_double)), math.nan)
    assert math.isnan(w[names.index("P")]) and w[names.index("NO3")] == 0.0
