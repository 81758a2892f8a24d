"""The library's fused PISCES functor, evaluated on the host in FP64, against the oracle's
per-tracer functors; default parameters byte-identical to the oracle's restatement."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from obgc import _abi as A
from test_oracle_pisces import INITIAL, conservation_case


def lib_point(p, values, aux, z, t):
    v = np.ascontiguousarray(values, dtype=np.float64)
    a = np.ascontiguousarray(aux, dtype=np.float64)
    G = np.zeros(A.PISCES_NUM_BGC)
    P = C.POINTER(C.c_double)
    A.check(A.load().obgc_pisces_eval_point(C.byref(p), v.ctypes.data_as(P), a.ctypes.data_as(P), z, t,
                                            G.ctypes.data_as(P)), "obgc_pisces_eval_point")
    return G


def random_state(rng):
    v = np.array([INITIAL.get(n, 0.0) for n in A.PISCES_ASCII], dtype=np.float64)
    v[:24] *= np.exp(rng.normal(0, 0.5, 24))
    v[A.PISCES_INDEX["T"]] = rng.uniform(2, 25)
    aux = np.array([rng.uniform(-150, -10), rng.uniform(-200, -20), 7.5, rng.uniform(0.5, 4), rng.uniform(0.1, 3),
                    rng.uniform(0, 200), -2 / 86400 * rng.uniform(0.5, 1), -rng.uniform(30, 200) / 86400,
                    rng.uniform(0, 300), rng.uniform(0, 100), rng.uniform(0, 100), rng.uniform(0, 100)])
    return v, aux, rng.uniform(-300, -1), rng.uniform(0, 3e7)


def test_defaults_match_the_oracle_bytes():
    a, b = A.PiscesParams(), O.pisces_defaults()
    A.check(A.load().obgc_pisces_default_params(C.byref(a)), "defaults")
    assert bytes(a) == bytes(b)


def test_conservation_case_matches_oracle():
    p, aux = conservation_case()
    v = [INITIAL.get(n, 0.0) for n in A.PISCES_ASCII]
    a = [aux[n] for n in A.PISCES_AUX]
    got = lib_point(p, v, a, -5.0, 0.0)
    ref = O.pisces_tendencies(p, v, a, -5.0, 0.0)
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-25)


@pytest.mark.parametrize("seed", range(8))
def test_random_states_match_oracle(seed):
    rng = np.random.default_rng(seed)
    p = O.pisces_defaults()
    for _ in range(20):
        v, a, z, t = random_state(rng)
        got = lib_point(p, v, a, z, t)
        ref = O.pisces_tendencies(p, v, a, z, t)
        scale = np.maximum(np.abs(ref), 1e-12 * np.max(np.abs(ref)))
        assert np.max(np.abs(got - ref) / scale) < 1e-10, dict(zip(A.PISCES_ASCII, (got - ref) / scale))


def test_zero_state_is_zero_on_the_library_path():
    p, aux = conservation_case()
    got = lib_point(p, np.zeros(26), [aux[n] for n in A.PISCES_AUX], -5.0, 0.0)
    assert np.all(got == 0.0)
