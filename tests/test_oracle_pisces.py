"""The oracle's PISCES against the reference's own tests (test/test_PISCES.jl): zero state stays zero,
element conservation of the tendencies (C, Fe, P, Si, N) at the reference's tolerances, mixed-layer
means and euphotic depth, and the negative-tracer scaling sequence."""
import math

import numpy as np
import pytest

import oracle as O
from obgc import _abi as A

# PISCES_INITIAL_VALUES (test/test_PISCES.jl:8-16)
INITIAL = dict(P=0.5, PChl=0.02, PFe=0.005, D=0.1, DChl=0.004, DFe=0.001, DSi=0.01, Z=0.1, M=0.7, DOC=2.1,
               POC=7.8, SFe=0.206, GOC=38, BFe=1.1, PSi=0.1, CaCO3=1e-10, NO3=2.3, NH4=0.9, PO4=0.6, Fe=0.13, Si=8.5,
               DIC=2205, Alk=2566, O2=317, T=10, S=35)


def conservation_case():
    """test_PISCES_conservation (test/test_PISCES.jl:33-64): box at z = -5, PAR1..3 = 100, PAR = 300,
    zmxl = zeu = -10, kappa = 1, mixed-layer PAR = 300, no sinking, no permanent iron removal, no
    nitrogen fixation."""
    p = O.pisces_defaults()
    p.excess_scavenging_enhancement = 0.0
    p.maximum_fixation_rate = 0.0
    p.poc_sinking_speed = 0.0
    aux = dict(zmxl=-10.0, zeu=-10.0, Si_clim=7.5, Omega=1.0, kappa=1.0, mixed_layer_PAR=300.0, wPOC=0.0, wGOC=0.0,
               PAR=300.0, PAR1=100.0, PAR2=100.0, PAR3=100.0)
    return p, aux


def test_zero_state_has_zero_tendencies():
    p, aux = conservation_case()
    G = O.pisces_tendencies(p, {}, aux, z=-5.0, t=0.0)
    assert np.all(G == 0.0), dict(zip(A.PISCES_TRACERS, G))


@pytest.mark.parametrize("t", [0.0, 1.0, 0.5 * 86400, 200 * 86400])
def test_element_conservation_of_tendencies(t):
    p, aux = conservation_case()
    G = O.pisces_tendencies(p, INITIAL, aux, z=-5.0, t=t)
    assert np.all(np.isfinite(G))
    names = A.PISCES_TRACERS
    groups = O.pisces_conserved_groups(p)
    # carbon, iron, phosphate, silicon, nitrogen and the reference's absolute tolerances
    tolerances = [1e-20, 1e-21, 1e-22, 1e-21, 1e-21]
    labels = ["carbon", "iron", "phosphate", "silicon", "nitrogen"]
    for (slots, factors), tol, label in zip(groups, tolerances, labels):
        total = sum(G[s] * f for s, f in zip(slots, factors))
        assert abs(total) <= tol, (label, total, [names[s] for s in slots])
    assert np.max(np.abs(G)) > 0


def test_conserved_groups_follow_coupling_utils():
    p = O.pisces_defaults()
    g = O.pisces_conserved_groups(p)
    names = [[A.PISCES_ASCII[s] for s in slots] for slots, _ in g]
    assert names[0] == ["P", "D", "Z", "M", "DOC", "POC", "GOC", "DIC", "CaCO3"]
    assert names[1] == ["PFe", "DFe", "Z", "M", "SFe", "BFe", "Fe"]
    assert g[1][1] == [1, 1, 0.01, 0.015, 1, 1, 1]
    assert names[2][-1] == "PO4" and g[2][1][0] == pytest.approx(1 / 122)
    assert names[3] == ["DSi", "Si", "PSi"]
    assert names[4][:2] == ["NH4", "NO3"] and g[4][1][2] == pytest.approx(16 / 122)


def test_mixed_layer_means():
    # test_PISCES_update_state (test/test_PISCES.jl:70-100): 10 levels over 100 m, PAR = 3 exp(z / 10),
    # kappa = 2 above -25 m and 1 below, mixed-layer depth -25
    Nz = 10
    zf = np.linspace(-100, 0, Nz + 1)
    zc = 0.5 * (zf[1:] + zf[:-1])
    PAR = 3 * np.exp(zc / 10)
    kappa = np.where(zc > -25, 2.0, 1.0)
    assert O.mixed_layer_mean(zf, PAR, -25.0) == pytest.approx(3 * 10 / 25 * (1 - math.exp(-25 / 10)), rel=0.1)
    assert O.mixed_layer_mean(zf, kappa, -25.0) == pytest.approx(2.0, rel=0.1)


def test_goc_sinking_speed_profile():
    p = O.pisces_defaults()
    zc = np.linspace(-995, -5, 100)
    w = O.goc_speed(p, zc, -50.0, -80.0)
    assert w[-1] == 0.0
    assert w[99] == pytest.approx(-30 / 86400)                       # within the mixed layer
    assert w[0] == pytest.approx(-30 / 86400 + (170 / 86400) * (-995 + 80) / 5000)


def scale(values, groups):
    gn, gs, gf = O.group_arrays(groups)
    v = np.array(values, dtype=np.float64)
    P = O.C.POINTER
    O.lib().or_scale_cell(v.ctypes.data_as(P(O.C.c_double)), 1, len(groups), gn.ctypes.data_as(P(O.C.c_int32)),
                          gs.ctypes.data_as(P(O.C.c_int32)), gf.ctypes.data_as(P(O.C.c_double)), math.nan)
    return v


def test_negativity_protection_sequence():
    # test_PISCES_negativity_protection (test/test_PISCES.jl:102-137)
    groups = O.pisces_conserved_groups(O.pisces_defaults())
    idx = A.PISCES_INDEX
    v = np.zeros(A.PISCES_NUM_BGC + 2)
    for n, x in dict(P=-1, D=1, Z=1, M=1, DOC=1, POC=1, GOC=1, DIC=1, CaCO3=1, PO4=1).items():
        v[idx[n]] = x
    v = scale(v, groups)
    assert v[idx["P"]] == 0
    for n in ("D", "Z", "M", "DOC", "POC", "GOC", "DIC", "CaCO3"):
        assert v[idx[n]] == pytest.approx(7 / 8)
    assert v[idx["PO4"]] == 1
    v[idx["Si"]], v[idx["DSi"]] = -1, 0.1
    v = scale(v, groups)
    assert math.isnan(v[idx["DSi"]])
    v[idx["Fe"]], v[idx["Z"]], v[idx["M"]] = -1, 1000, 0
    v = scale(v, groups)
    assert v[idx["Fe"]] == 0
    assert v[idx["Z"]] == pytest.approx(900)
