"""The oracle's carbon chemistry against the reference's known answers.

Values and tolerances are those of test/test_gasexchange_carbon_chem.jl:259-301 (Dickson et al.
2007; Zeebe & Wolf-Gladrow 2001), :314-327 (virial coefficients, pCO2 = 350 +- 0.1) and the
CarbonChemistry doctest (src/Models/CarbonChemistry/carbon_chemistry.jl:55-62).
"""
import math

import pytest

import oracle as O
from obgc import _abi as A

S, TK, P = 35, 298.15, 300


@pytest.mark.parametrize("which,fn,value,atol", [
    (O.K0, math.log, -3.5617, 1e-4),
    (O.K1, math.log10, -5.8472, 1e-4),
    (O.K2, math.log10, -8.9660, 1e-4),
    (O.KB, math.log, -19.7964, 1e-4),
    (O.KW, math.log, -30.434, 1e-3),
    (O.KS, math.log, -2.30, 1e-2),
    (O.KF, math.log, -6.09, 1e-2),
    (O.KP1, math.log, -3.71, 1e-2),
    (O.KP2, math.log, -13.727, 1e-3),
    (O.KP3, math.log, -20.24, 1e-2),
    (O.KSI, math.log, -21.61, 1e-2),
    (O.KSP_ARAGONITE, math.log10, -6.1883, 1e-4),
    (O.KSP_CALCITE, math.log10, -6.3693, 1e-4),
])
def test_equilibrium_constants(which, fn, value, atol):
    assert abs(fn(O.K(which, TK, S)) - value) <= atol


@pytest.mark.parametrize("which,value", [
    (O.K1, 1.30804), (O.K2, 1.21341), (O.KB, 1.38024), (O.KW, 1.23784), (O.KS, 1.21844),
    (O.KF, 1.13151), (O.KP1, 1.14852), (O.KP2, 1.27298), (O.KP3, 1.32217),
    (O.KSP_ARAGONITE, 1.47866), (O.KSP_CALCITE, 1.52962),
])
def test_pressure_corrections(which, value):
    assert abs(O.pressure_correction(which, TK, P) - value) <= 1e-5


def test_virial_coefficients():
    L = O.lib()
    assert abs(L.or_first_virial(25 + 273.15) - (-123.2e-6)) <= 1e-8
    assert abs(L.or_cross_virial(25 + 273.15) - 22.5e-6) <= 1e-7


def test_pco2_350():
    # test_gasexchange_carbon_chem.jl:319-327
    pco2 = O.carbon_chemistry(2136.242890518708, 25.0, 35.0, Alk=2500.0, output=A.OUT_PCO2)
    assert abs(pco2 - 350) <= 0.1
    # and with EOS-80 standing in, as the oracle did before the polynomial was restated
    pco2 = O.carbon_chemistry(2136.242890518708, 25.0, 35.0, Alk=2500.0, output=A.OUT_PCO2, density="eos80")
    assert abs(pco2 - 350) <= 0.1


def doctest_density():
    """Density implied by doctest 3 (pH given: fCO2 is linear in 1/rho)."""
    H = 10.0 ** -7.5
    Tk = 10.0 + 273.15
    K1, K2, K0 = (O.K(w, Tk, 35.0) for w in (O.K1, O.K2, O.K0))
    f = 2000.0 * 1e-3 * H * H / (H * H + K1 * H + K1 * K2) / K0 * 1e6
    return f / 1315.7136384737507


def test_doctest_digits_at_the_default_density():
    # the default density (the TEOS-10 polynomial of Roquet et al. 2015, evaluated as
    # seawater_density.jl:33-39 evaluates it, at the functor's default P = 1 bar) reproduces the
    # three doctest digits of carbon_chemistry.jl:55-62
    f1 = O.carbon_chemistry(2000.0, 10.0, 35.0, Alk=2000.0)
    ph = O.carbon_chemistry(2000.0, 10.0, 35.0, Alk=2000.0, output=A.OUT_PH_FREE)
    f3 = O.carbon_chemistry(2000.0, 10.0, 35.0, pH=7.5)
    assert f1 == pytest.approx(1308.1474527899106, rel=1e-14, abs=0)
    assert ph == pytest.approx(7.502532746463654, rel=1e-14, abs=0)
    assert f3 == pytest.approx(1315.7136384737507, rel=1e-14, abs=0)
    # the density itself: the one the third digit implies (fCO2 is linear in 1 / rho there)
    assert O.density_teos10_polynomial(10.0, 35.0, 1.0) == pytest.approx(doctest_density(), rel=1e-14, abs=0)


def test_teos10_polynomial_against_eos80():
    # the two equations of state agree to the size of the practical / absolute salinity and
    # temperature-scale differences (<= 0.2 kg/m3 over the ocean's range at the surface)
    for T in (-1.0, 5.0, 15.0, 25.0, 30.0):
        for S in (30.0, 35.0, 38.0):
            assert abs(O.density_teos10_polynomial(T, S, 0.0) - O.density_eos80(T, S, 0.0)) < 0.2
    # the reference's Z = +10 m per bar makes the polynomial's height positive: density falls with P
    assert O.density_teos10_polynomial(10.0, 35.0, 100.0) < O.density_teos10_polynomial(10.0, 35.0, 0.0)


def test_doctest_digits_with_implied_density():
    rho = doctest_density()
    # 1e-3 of EOS-80: the doctest density is a plausible seawater density at 10 degC, 35 psu
    assert abs(rho - O.density_eos80(10.0, 35.0, 1.0)) < 0.5
    f1 = O.carbon_chemistry(2000.0, 10.0, 35.0, Alk=2000.0, density=rho)
    ph = O.carbon_chemistry(2000.0, 10.0, 35.0, Alk=2000.0, density=rho, output=A.OUT_PH_FREE)
    f3 = O.carbon_chemistry(2000.0, 10.0, 35.0, pH=7.5, density=rho)
    assert f1 == pytest.approx(1308.1474527899106, rel=1e-14, abs=0)
    assert ph == pytest.approx(7.502532746463654, rel=1e-14, abs=0)
    assert f3 == pytest.approx(1315.7136384737507, rel=1e-14, abs=0)


def test_eos80_check_values():
    # UNESCO (1981) check values
    assert O.density_eos80(5, 0, 0) == pytest.approx(999.96675, abs=5e-5)
    assert O.density_eos80(5, 35, 0) == pytest.approx(1027.67547, abs=5e-5)
    assert O.density_eos80(25, 35, 1000) == pytest.approx(1062.53817, abs=5e-5)


def test_outputs_consistent():
    rho = doctest_density()
    H = O.carbon_chemistry(2100.0, 12.0, 35.0, Alk=2350.0, density=rho, output=A.OUT_H)
    phf = O.carbon_chemistry(2100.0, 12.0, 35.0, Alk=2350.0, density=rho, output=A.OUT_PH_FREE)
    pht = O.carbon_chemistry(2100.0, 12.0, 35.0, Alk=2350.0, density=rho, output=A.OUT_PH_TOTAL)
    phs = O.carbon_chemistry(2100.0, 12.0, 35.0, Alk=2350.0, density=rho, output=A.OUT_PH_SWS)
    assert phf == pytest.approx(-math.log10(H), rel=1e-15)
    assert phs < pht < phf      # total and seawater scales add HSO4 (and HF): lower pH
    f = O.carbon_chemistry(2100.0, 12.0, 35.0, Alk=2350.0, density=rho)
    p = O.carbon_chemistry(2100.0, 12.0, 35.0, Alk=2350.0, density=rho, output=A.OUT_PCO2)
    assert p > f and abs(p / f - 1) < 0.01   # fugacity below partial pressure by < 1%
    om = O.carbon_chemistry(2100.0, 12.0, 35.0, Alk=2350.0, output=A.OUT_OMEGA)
    assert 1.0 < om < 10.0
