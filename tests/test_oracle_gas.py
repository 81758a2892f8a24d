"""Oracle (CPU restatement) of the air-sea gas exchange against the reference's known answers:
test/test_gasexchange_carbon_chem.jl:157-193 (Schmidt numbers at 20 degC from Wanninkhof 2014,
pCO2 = 350 +- 0.1 from Dickson et al. 2007, oxygen air concentration 'ball park' 200 +- 50)."""
import numpy as np
import pytest

import oracle as O
from obgc import _abi as A


def test_schmidt_numbers_wanninkhof_2014():
    co2, o2 = O.gas_exchange_defaults(A.GAS_CO2), O.gas_exchange_defaults(A.GAS_O2)
    assert O.schmidt_number(co2, 20.0) == pytest.approx(668, abs=1)
    assert O.schmidt_number(o2, 20.0) == pytest.approx(568, abs=1)


def test_co2_water_concentration_is_dickson_pco2():
    # flux = k (pCO2 - air): with air = 350 ppmv the flux vanishes to the pCO2 = 350 +- 0.1 of the test
    g = O.gas_exchange_defaults(A.GAS_CO2)
    k = O.gas_exchange_flux(g, 25.0, 35.0, DIC=2136.242890518708, Alk=2500.0, air=349.0) - \
        O.gas_exchange_flux(g, 25.0, 35.0, DIC=2136.242890518708, Alk=2500.0, air=350.0)
    assert k > 0
    pco2 = 350.0 + O.gas_exchange_flux(g, 25.0, 35.0, DIC=2136.242890518708, Alk=2500.0, air=350.0) / k
    assert pco2 == pytest.approx(350, abs=0.1)


def test_oxygen_air_concentration_ball_park():
    g = O.gas_exchange_defaults(A.GAS_O2)
    assert g.air_concentration * O.o2_solubility(g, 25.0, 35.0) == pytest.approx(200, abs=50)


def test_transfer_velocity_ho06_and_sign():
    # k660 = 0.266 / hour / 100 u^2 (gas_transfer_velocity.jl:53-59), scaled by sqrt(660 / Sc)
    g = O.gas_exchange_defaults(A.GAS_O2)
    T, S, O2, u = 12.0, 34.0, 300.0, 7.0
    air = g.air_concentration * O.o2_solubility(g, T, S)
    k = 0.266 / 3600 / 100 * u ** 2 / np.sqrt(O.schmidt_number(g, T) / 660)
    assert O.gas_exchange_flux(g, T, S, O2=O2, u10=u) == pytest.approx(k * (O2 - air), rel=1e-14)
    # supersaturated water outgasses (positive, out of the ocean)
    assert O.gas_exchange_flux(g, T, S, O2=2 * air, u10=u) > 0
    assert O.gas_exchange_flux(g, T, S, O2=0.5 * air, u10=u) < 0


@pytest.mark.parametrize("air", [413.1, 413.0])
def test_replicated_carbonate_systems_surface_flux(air):
    # test/test_gasexchange_carbon_chem.jl:21-67: T = 15, S = 35, the default wind; DIC 2220 / Alk
    # 2500 gives a surface flux of -8e-6 +- 1e-6 (into the ocean), and the second replicate (2221 /
    # 2501) another value of the same size
    g = O.gas_exchange_defaults(A.GAS_CO2)
    f1 = O.gas_exchange_flux(g, 15.0, 35.0, DIC=2220.0, Alk=2500.0, air=air)
    f2 = O.gas_exchange_flux(g, 15.0, 35.0, DIC=2221.0, Alk=2501.0, air=air)
    assert f1 == pytest.approx(-8e-6, abs=1e-6)
    assert f2 == pytest.approx(-8e-6, abs=1e-6)
    assert f1 != f2
