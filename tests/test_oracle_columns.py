"""The oracle's column runner (CPU): conservation with a closed bottom, the alkalinity pulse, and
independence of columns run in one call.  These pin the column path's host semantics; the GPU
engine is compared with this runner in test_gpu_columns.py."""
import numpy as np

import obgc
import oracle as O


def run(bgc, cols, names):
    nt = len(names)
    so, ko, s, k, specs = [], [], [], [], []
    a = b = 0
    for c in cols:
        Nz = c["init"].shape[1]
        so.append(a)
        ko.append(b)
        s.append(c["init"].ravel())
        k.append(c["kappa"])
        a += nt * Nz
        b += Nz + 1
        specs.append(O.Column(Nz, c["nsteps"], c["dz"], c["surface_PAR"], c.get("mu0", 0.0), c["dt"],
                              c.get("pulse_step", -1), c.get("pulse_k", -1), c.get("pulse_amount", 0.0)))
    state = np.concatenate(s)
    O.columns_run(bgc.params, obgc._abi.default_twoband(), specs, names, state, np.concatenate(k), so, ko, 0.0, 0)
    return [state[so[q]:so[q] + nt * c["init"].shape[1]].reshape(nt, -1) for q, c in enumerate(cols)]


def test_npzd_nitrogen_is_conserved_with_a_closed_bottom():
    bgc = obgc.NPZD(None)
    bgc.params.open_bottom = 0
    cols = obgc.npzd_column_ensemble(6, seed=2, levels=(16, 64), nsteps=40)
    names = obgc.required_biogeochemical_tracers(bgc)
    out = run(bgc, cols, names)
    rows = [names.index(n) for n in ("N", "P", "Z", "D")]
    for c, o in zip(cols, out):
        before = c["init"][rows].sum()
        after = o[rows].sum()
        assert abs(after - before) < 1e-12 * before
        assert np.max(np.abs(o - c["init"])) > 1e-4


def test_lobster_pulse_adds_exactly_its_alkalinity():
    bgc = obgc.LOBSTER(None, carbonate_system=obgc.CarbonateSystem())
    names = obgc.required_biogeochemical_tracers(bgc)
    rng = np.random.default_rng(4)
    c = obgc.lobster_column_request(rng, levels=(24, 40), days=(0.5, 0.5))
    c["pulse_step"], c["pulse_k"], c["pulse_amount"] = 3, c["init"].shape[1] - 2, 250.0
    quiet = dict(c, pulse_amount=0.0)
    with_pulse, without = run(bgc, [c, quiet], names)
    ialk = names.index("Alk")
    others = [q for q in range(len(names)) if q != ialk]
    assert np.array_equal(with_pulse[others], without[others])       # Alk feeds back into nothing
    added = (with_pulse[ialk] - without[ialk]).sum()
    assert abs(added - 250.0) < 1e-9 * 2400 * c["init"].shape[1]
    assert np.max(np.abs(with_pulse[ialk] - without[ialk])) < 250.0   # spread by diffusion


def test_columns_are_independent_in_one_call():
    bgc = obgc.NPZD(None)
    cols = obgc.npzd_column_ensemble(5, seed=7, levels=(16, 80), nsteps=15)
    names = obgc.required_biogeochemical_tracers(bgc)
    together = run(bgc, cols, names)
    for c, t in zip(cols, together):
        assert np.array_equal(run(bgc, [c], names)[0], t)


def test_co2_exchange_column_equals_the_3d_step_of_a_single_column():
    """The column runner's CO2 condition (examples/column.jl:54-64) against the oracle's 3-D step of a
    1 x 1 x Nz grid carrying the same T and S as tracers, with no diffusion: the two restatements of
    the top boundary condition agree to rounding."""
    bgc = obgc.LOBSTER(None, carbonate_system=obgc.CarbonateSystem())
    rng = np.random.default_rng(4)
    c = obgc.lobster_column_request(rng, levels=(24, 24), days=(0.5, 0.5), pulse=(300.0, 300.0))
    c["kappa"] = np.zeros_like(c["kappa"])
    names = list(obgc.required_biogeochemical_tracers(bgc))
    co2 = O.gas_exchange_defaults(obgc._abi.GAS_CO2)
    co2.wind_speed = 9.0
    Nz, nt = c["init"].shape[1], len(names)
    spec = O.Column(Nz, c["nsteps"], c["dz"], c["surface_PAR"], 0.0, c["dt"], -1, -1, 0.0, c["T"], c["S"])
    col = np.ascontiguousarray(c["init"].ravel().copy())
    O.columns_run(bgc.params, obgc._abi.default_twoband(), [spec], names, col, c["kappa"], [0], [0], 0.0, 0, gas=co2)
    g = obgc.RectilinearGrid((1, 1, Nz), (1.0, 1.0, Nz * c["dz"]), ("Flat", "Flat", "Bounded"))
    m = O.model3d(bgc.params, g.c_grid(), names + ["T", "S"], surface_kind=obgc._abi.SURFACE_CONSTANT,
                  surface_value=c["surface_PAR"], gas_exchange=[co2])
    s3 = np.concatenate([c["init"], np.full((1, Nz), c["T"]), np.full((1, Nz), c["S"])]).reshape(nt + 2, Nz, 1, 1)
    s3 = np.ascontiguousarray(s3)
    O.step3d(m, s3, t=0.0, dt=c["dt"], nsteps=c["nsteps"])
    col = col.reshape(nt, Nz)
    for q in range(nt):
        assert np.max(np.abs(col[q] - s3[q, :, 0, 0])) <= 1e-12 * np.max(np.abs(s3[q])), names[q]
    # and the condition did something: the surface DIC differs from a run without it
    plain = np.ascontiguousarray(c["init"].ravel().copy())
    O.columns_run(bgc.params, obgc._abi.default_twoband(), [spec], names, plain, c["kappa"], [0], [0], 0.0, 0)
    q = names.index("DIC")
    assert abs(plain.reshape(nt, Nz)[q, -1] - col[q, -1]) > 1e-2


def test_implicit_vertical_diffusion_of_the_3d_step_equals_the_column_runner():
    """VerticallyImplicitTimeDiscretization in the oracle's 3-D step (a 1 x 1 x Nz grid) against the
    column runner, whose vertical diffusion has always been implicit: equal to rounding."""
    bgc = obgc.LOBSTER(None, carbonate_system=obgc.CarbonateSystem())
    rng = np.random.default_rng(8)
    c = obgc.lobster_column_request(rng, levels=(30, 30), days=(0.5, 0.5))
    names = list(obgc.required_biogeochemical_tracers(bgc))
    Nz, nt = c["init"].shape[1], len(names)
    spec = O.Column(Nz, c["nsteps"], c["dz"], c["surface_PAR"], 0.0, c["dt"], -1, -1, 0.0, c["T"], c["S"])
    col = np.ascontiguousarray(c["init"].ravel().copy())
    O.columns_run(bgc.params, obgc._abi.default_twoband(), [spec], names, col, c["kappa"], [0], [0], 0.0, 0)
    g = obgc.RectilinearGrid((1, 1, Nz), (1.0, 1.0, Nz * c["dz"]), ("Flat", "Flat", "Bounded"))
    m = O.model3d(bgc.params, g.c_grid(), names, surface_kind=obgc._abi.SURFACE_CONSTANT, surface_value=c["surface_PAR"],
                  kappa_z_faces=c["kappa"], vertical_implicit=True)
    s3 = np.ascontiguousarray(c["init"].reshape(nt, Nz, 1, 1).copy())
    O.step3d(m, s3, t=0.0, dt=c["dt"], nsteps=c["nsteps"])
    col = col.reshape(nt, Nz)
    for q in range(nt):
        assert np.max(np.abs(col[q] - s3[q, :, 0, 0])) <= 1e-12 * np.max(np.abs(s3[q])), names[q]
    assert np.max(np.abs(c["kappa"])) >= 1e-3      # a mixed layer: explicit steps of this dt would be unstable
