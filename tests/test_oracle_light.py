"""The oracle's light models against the closed forms of test/test_light.jl:12-106."""
import numpy as np
import pytest

import oracle as O
from obgc import _abi as A


def grid_z(Nz, Lz):
    dz = Lz / Nz
    zf = -Lz + dz * np.arange(Nz + 1)
    return zf[:-1] + dz / 2, zf


def test_two_band_closed_form():
    # test_light.jl:12-50: 2x2x2 grid, extent 2, P = 2.5 + z, surface PAR 100
    lp = A.default_twoband()
    zc, zf = grid_z(2, 2.0)
    P = 2.5 + zc
    got = O.twoband_column(lp, zc, zf, P, 100.0)
    kr, kb, xr, xb = lp.water_red_attenuation, lp.water_blue_attenuation, lp.chlorophyll_red_attenuation, lp.chlorophyll_blue_attenuation
    er, eb, r, Rc = lp.chlorophyll_red_exponent, lp.chlorophyll_blue_exponent, lp.pigment_ratio, lp.phytoplankton_chlorophyll_ratio
    ir = [(2.0 * Rc / r) ** er * 0.5]
    ib = [(2.0 * Rc / r) ** eb * 0.5]
    ir.append(ir[0] + (2.0 * Rc / r) ** er * 0.5 + (1.0 * Rc / r) ** er * 0.5)
    ib.append(ib[0] + (2.0 * Rc / r) ** eb * 0.5 + (1.0 * Rc / r) ** eb * 0.5)
    expected = 100.0 * np.array([np.exp(-0.5 * kr - ir[0] * xr) + np.exp(-0.5 * kb - ib[0] * xb),
                                 np.exp(-1.5 * kr - ir[1] * xr) + np.exp(-1.5 * kb - ib[1] * xb)]) / 2
    np.testing.assert_allclose(got, expected[::-1], rtol=1.5e-8)


def test_multi_band_single():
    # test_light.jl:53-72: one band (1, 2) nm with flat coefficients, Chl = 2
    kw, e, chi = O.multiband_coefficients([(1, 2)], [1, 2], [0.01, 0.01], [2, 2], [0.1, 0.1])
    assert kw[0] == pytest.approx(0.01) and e[0] == pytest.approx(2) and chi[0] == pytest.approx(0.1)
    zc, _ = grid_z(2, 2.0)
    Chl = np.full(2, 1.31 * (2 / 1.31))
    got = O.multiband_column(zc, kw[0], e[0], chi[0], Chl, 100.0 * 1.0)
    np.testing.assert_allclose(got, 100 * np.exp(zc * (0.01 + 0.1 * 2 ** 2)), rtol=1.5e-8)


def test_multi_band_two_bands():
    # test_light.jl:74-100
    kw, e, chi = O.multiband_coefficients([(1, 2), (8, 9)], [1, 2, 8, 9], [0.01, 0.01, 0.02, 0.02],
                                          [2, 2, 1.5, 1.5], [0.1, 0.1, 0.2, 0.2])
    zc, _ = grid_z(2, 2.0)
    Chl = np.full(2, 1.31 * (2 / 1.31))
    p1 = O.multiband_column(zc, kw[0], e[0], chi[0], Chl, 100.0 * 0.5)
    p2 = O.multiband_column(zc, kw[1], e[1], chi[1], Chl, 100.0 * 0.5)
    e1 = 100 * np.exp(zc * (0.01 + 0.1 * 2 ** 2)) / 2
    e2 = 100 * np.exp(zc * (0.02 + 0.2 * 2 ** 1.5)) / 2
    np.testing.assert_allclose(p1, e1, atol=1e-4)
    np.testing.assert_allclose(p2, e2, atol=1e-4)
    np.testing.assert_allclose(p1 + p2, e1 + e2, atol=1e-3)


def test_default_surface_par():
    # Light.jl:45-47
    assert O.default_surface_PAR(0.0) == 100.0
    assert O.default_surface_PAR(6 * 3600.0) == pytest.approx(0.0, abs=1e-12)
    assert O.default_surface_PAR(12 * 3600.0) == 0.0
    assert O.default_surface_PAR(3 * 3600.0) == pytest.approx(100 * np.cos(np.pi / 4))


def test_euphotic_depth_exponential_profile():
    # A PAR = PAR0 exp(z/10) profile crosses 1e-3 of the surface value at z = -10 ln(1000)
    # (the known answer of test/test_PISCES.jl:98-112).
    Nz, Lz = 400, 200.0
    zc, _ = grid_z(Nz, Lz)
    PAR = 100 * np.exp(zc / 10)
    halo_above = 100 * np.exp((zc[-1] + Lz / Nz) / 10)
    zc_h = np.append(zc, zc[0] - Lz / Nz)
    zeu = O.euphotic_depth_column(zc_h, PAR, halo_above, 1e-3)
    assert zeu == pytest.approx(-10 * np.log(1000), abs=1e-2)
