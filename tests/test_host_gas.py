"""Air-sea gas exchange: the library's device function, called on the host through
obgc_gas_exchange_point, against the oracle (no GPU), and the defaults struct byte for byte."""
import ctypes as C

import numpy as np
import pytest

import obgc
import oracle as O
from obgc import _abi as A


@pytest.mark.parametrize("gas", [A.GAS_CO2, A.GAS_O2])
def test_defaults_match_oracle_bytes(gas):
    lib_g = obgc.GasExchange(gas).params
    ref = O.gas_exchange_defaults(gas)
    assert bytes(lib_g) == bytes(ref)


@pytest.mark.parametrize("gas", [A.GAS_CO2, A.GAS_O2])
def test_point_flux_matches_oracle(gas):
    g = obgc.GasExchange(gas)
    ref = O.gas_exchange_defaults(gas)
    rng = np.random.default_rng(gas)
    worst = 0.0
    for _ in range(200):
        T, S = rng.uniform(-1, 30), rng.uniform(30, 38)
        DIC, Alk = rng.uniform(1900, 2300), rng.uniform(2200, 2500)
        O2 = rng.uniform(150, 350)
        u = rng.uniform(0, 20)
        air = rng.uniform(300, 600) if gas == A.GAS_CO2 else rng.uniform(8000, 10000)
        got = g(T, S, DIC=DIC, Alk=Alk, O2=O2, u10=u, air=air)
        want = O.gas_exchange_flux(ref, T, S, DIC=DIC, Alk=Alk, O2=O2, u10=u, air=air)
        worst = max(worst, abs(got - want) / max(abs(want), 1e-30))
    assert worst < 1e-11


def test_custom_coefficients_reach_the_device_struct():
    # Wanninkhof14 k660 and a constant-1 Schmidt number: k = 0.251/hour/100 u^2 sqrt(660)
    g = obgc.OxygenGasExchangeBoundaryCondition(k660=(0, 0, 0.251 / 3600 / 100), schmidt=(1.0,), wind_speed=5.0,
                                               air_concentration=0.0)
    assert g(10.0, 35.0, O2=200.0) == pytest.approx(0.251 / 3600 / 100 * 25 * np.sqrt(660) * 200, rel=1e-13)
    with pytest.raises(ValueError):
        obgc.GasExchange(A.GAS_CO2, k660=(1, 2, 3, 4, 5))
