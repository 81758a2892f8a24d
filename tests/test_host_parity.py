"""Host-compiled product code (libobgc.so, no GPU needed) against the oracle: model presets, tracer
lists, drift velocities, the fused continuous-form functor and the FP64 carbonate solve."""
import itertools
import math

import numpy as np
import pytest

import obgc
import oracle as O
from obgc import _abi as A

from test_oracle_npd import ALL, initial_values


def test_presets_match_oracle_bytes():
    for name in ("LOBSTER", "NPZD"):
        assert bytes(obgc.preset(name)) == bytes(O.preset(name))


def test_required_tracers_all_configs():
    g = obgc.RectilinearGrid((4, 4, 8), (1.0, 1.0, 8.0))
    for _, p in ALL:
        bgc = obgc.LOBSTER(g)
        bgc.params = p
        assert [A.NAME_INDEX[n] for n in obgc.required_biogeochemical_tracers(bgc)] == O.required_tracers(p)


def test_drift_velocity_profiles():
    g = obgc.RectilinearGrid((4, 4, 10), (1.0, 1.0, 20.0))
    for open_bottom in (0, 1):
        for base in ("LOBSTER", "NPZD"):
            bgc = obgc.LOBSTER(g) if base == "LOBSTER" else obgc.NPZD(g)
            bgc.params.open_bottom = open_bottom
            for name in obgc.required_biogeochemical_tracers(bgc):
                got = obgc.biogeochemical_drift_velocity(bgc, name)
                ref = O.drift_profile(bgc.params, name, 10)
                if ref is None:
                    assert got is None
                else:
                    np.testing.assert_array_equal(got, ref)
                    assert got[-1] == 0.0


def test_fused_functor_matches_oracle_all_configs():
    rng = np.random.default_rng(11)
    g = obgc.RectilinearGrid((1, 1, 1), (1.0, 1.0, 1.0))
    worst = 0.0
    for _, p in ALL:
        bgc = obgc.LOBSTER(g)
        bgc.params = p
        for trial in range(3):
            vals = initial_values(p, rng)
            PAR = float(rng.uniform(0, 300))
            for name in obgc.required_biogeochemical_tracers(bgc):
                got = obgc.eval_point(bgc, name, vals, PAR)
                ref = O.tendency(p, name, vals, PAR)
                scale = max(abs(ref), 1e-300)
                worst = max(worst, abs(got - ref) / scale if abs(ref) > 1e-14 else abs(got - ref))
    assert worst < 1e-12


def test_npzd_functor_with_temperature():
    g = obgc.RectilinearGrid((1, 1, 1), (1.0, 1.0, 1.0))
    bgc = obgc.NPZD(g)
    vals = {"N": 7.0, "P": 0.2, "Z": 0.05, "T": 14.0, "D": 0.3}
    for name in ("N", "P", "Z", "T", "D"):
        assert obgc.eval_point(bgc, name, vals, 55.0) == pytest.approx(O.tendency(bgc.params, name, vals, 55.0), rel=1e-13, abs=1e-30)


def test_zero_state_stays_finite_and_zero():
    g = obgc.RectilinearGrid((1, 1, 1), (1.0, 1.0, 1.0))
    for _, p in ALL:
        bgc = obgc.LOBSTER(g)
        bgc.params = p
        for name in obgc.required_biogeochemical_tracers(bgc):
            assert obgc.eval_point(bgc, name, {}, 100.0) == 0.0


@pytest.mark.parametrize("output", ["fCO2", "pCO2", "pHf", "pHt", "pHs", "Omega"])
def test_carbon_point_matches_oracle(output):
    cc = obgc.CarbonChemistry()
    rng = np.random.default_rng(3)
    for _ in range(40):
        DIC, Alk = rng.uniform(1900, 2300), rng.uniform(2150, 2500)
        T, S = rng.uniform(-1, 30), rng.uniform(30, 38)
        code = {"fCO2": A.OUT_FCO2, "pCO2": A.OUT_PCO2, "pHf": A.OUT_PH_FREE, "pHt": A.OUT_PH_TOTAL,
                "pHs": A.OUT_PH_SWS, "Omega": A.OUT_OMEGA}[output]
        got = cc(DIC, T, S, Alk=Alk, output=output)
        ref = O.carbon_chemistry(DIC, T, S, Alk=Alk, output=code)
        if output.startswith("pH"):
            assert abs(got - ref) <= 1e-12
        else:
            assert got == pytest.approx(ref, rel=1e-11)


def test_carbon_point_doctest_digits():
    # the library's own TEOS-10 polynomial (Horner form), the default density, gives the three
    # doctest digits of carbon_chemistry.jl:55-62 with no density supplied
    cc = obgc.CarbonChemistry()
    assert cc(2000.0, 10.0, 35.0, Alk=2000.0) == pytest.approx(1308.1474527899106, rel=1e-14)
    assert cc(2000.0, 10.0, 35.0, Alk=2000.0, output="pHf") == pytest.approx(7.502532746463654, rel=1e-14)
    assert cc(2000.0, 10.0, 35.0, pH=7.5) == pytest.approx(1315.7136384737507, rel=1e-14)
    # and so does a constant density equal to the one the third digit implies
    from test_oracle_carbon import doctest_density
    rho = doctest_density()
    cc = obgc.CarbonChemistry(density=rho)
    assert cc(2000.0, 10.0, 35.0, Alk=2000.0) == pytest.approx(1308.1474527899106, rel=1e-13)
    assert cc(2000.0, 10.0, 35.0, Alk=2000.0, output="pHf") == pytest.approx(7.502532746463654, rel=1e-14)
    assert cc(2000.0, 10.0, 35.0, pH=7.5) == pytest.approx(1315.7136384737507, rel=1e-13)
    assert obgc.CarbonChemistry()(2136.242890518708, 25.0, 35.0, Alk=2500.0, output="pCO2") == pytest.approx(350, abs=0.1)


def test_multiband_coefficients_match_oracle():
    bands = ((400, 500), (500, 600), (600, 700))
    got = obgc.light.numerical_mean_coefficients(bands)
    ref = O.multiband_coefficients(bands, obgc.light.MOREL_LAMBDA, obgc.light.MOREL_KW, obgc.light.MOREL_E, obgc.light.MOREL_CHI)
    for a, b in zip(got, ref):
        np.testing.assert_allclose(a, b, rtol=1e-15)
    with pytest.raises(ValueError):
        obgc.MultiBandPhotosyntheticallyActiveRadiation(surface_PAR_division=[0.5, 0.2, 0.2])


def test_aragonite_saturation_matches_oracle():
    # CarbonChemistry(calcite_solubility = KSP_aragonite()): Omega against aragonite, with and without
    # the depth pressure; the aragonite / calcite ratio is KSP_calcite / KSP_aragonite
    import oracle as O
    cc_a = obgc.CarbonChemistry(calcite_solubility="aragonite")
    cc_c = obgc.CarbonChemistry()
    for (DIC, Alk, T, S, P) in [(2100.0, 2350.0, 12.0, 35.0, None), (2200.0, 2400.0, 4.0, 34.5, 150.0)]:
        oa = cc_a(DIC, T, S, Alk=Alk, P=P, output="Omega")
        oc = cc_c(DIC, T, S, Alk=Alk, P=P, output="Omega")
        ref = O.carbon_chemistry(DIC, T, S, Alk=Alk, P=P, output=A.OUT_OMEGA, saturation_mineral=1)
        assert oa == pytest.approx(ref, rel=1e-12)
        Tk = T + 273.15
        ratio = O.K(O.KSP_CALCITE, Tk, S, P) / O.K(O.KSP_ARAGONITE, Tk, S, P)
        assert oa / oc == pytest.approx(ratio, rel=1e-12)
    with pytest.raises(ValueError):
        obgc.CarbonChemistry(calcite_solubility="dolomite")
