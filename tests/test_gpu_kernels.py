"""GPU parity: light, mode-(i) tendencies, carbonate solve, box models and the budget against the
oracle, through the C ABI (libobgc.so)."""
import ctypes as C
import math

import numpy as np
import pytest

import obgc
import oracle as O
from obgc import _abi as A
from gpuhelp import cuda, rel_err
from test_oracle_npd import ALL, initial_values

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype,tol", [("f64", 1e-13), ("f32", 2e-6)])
@pytest.mark.parametrize("surface", [None, 37.5])
def test_twoband_par(dtype, tol, surface):
    torch = cuda()
    g = obgc.RectilinearGrid((37, 5, 23), (1.0, 1.0, 115.0), dtype=dtype)
    rng = np.random.default_rng(1)
    P = rng.lognormal(np.log(0.3), 0.6, g.shape)
    td = torch.float64 if dtype == "f64" else torch.float32
    Pt = torch.as_tensor(P, dtype=td, device="cuda")
    PAR = torch.zeros_like(Pt)
    light = obgc.TwoBandPhotosyntheticallyActiveRadiation(grid=g, surface_PAR=surface)
    t = 3 * 3600.0
    light.compute(Pt, PAR, t=t)
    torch.cuda.synchronize()
    zc, zf = g.znodes(), g.znodes("face")
    PAR0 = surface if surface is not None else O.default_surface_PAR(t)
    ref = np.zeros(g.shape)
    Pin = Pt.double().cpu().numpy()
    for j in range(g.Ny):
        for i in range(g.Nx):
            ref[:, j, i] = O.twoband_column(light.params, zc, zf, Pin[:, j, i], PAR0)
    assert rel_err(PAR.cpu().numpy(), ref) < tol


@pytest.mark.parametrize("dtype,tol", [("f64", 1e-13), ("f32", 2e-6)])
def test_multiband_par_and_euphotic_depth(dtype, tol):
    torch = cuda()
    g = obgc.RectilinearGrid((9, 7, 40), (1.0, 1.0, 200.0), dtype=dtype)
    td = torch.float64 if dtype == "f64" else torch.float32
    rng = np.random.default_rng(2)
    Chl = torch.as_tensor(rng.lognormal(np.log(0.5), 0.5, g.shape), dtype=td, device="cuda")
    mb = obgc.MultiBandPhotosyntheticallyActiveRadiation(grid=g, surface_PAR=100.0)
    bands = [torch.zeros_like(Chl) for _ in range(3)]
    total = torch.zeros_like(Chl)
    mb.compute(Chl, bands, total)
    torch.cuda.synchronize()
    zc = g.znodes()
    C_ = Chl.double().cpu().numpy()
    tot_ref = np.zeros(g.shape)
    for b in range(3):
        ref = np.zeros(g.shape)
        for j in range(g.Ny):
            for i in range(g.Nx):
                ref[:, j, i] = O.multiband_column(zc, mb.kw[b], mb.e[b], mb.chi[b], C_[:, j, i], 100.0 * mb.division[b])
        assert rel_err(bands[b].cpu().numpy(), ref) < tol
        tot_ref += ref
    assert rel_err(total.cpu().numpy(), tot_ref) < tol
    # euphotic depth of an exponential profile crosses 1e-3 at -10 ln 1000 (test_PISCES.jl:98-124)
    g2 = obgc.RectilinearGrid((3, 2, 400), (1.0, 1.0, 200.0), dtype=dtype)
    z = g2.znodes()
    PAR = torch.as_tensor(np.broadcast_to(100 * np.exp(z / 10)[:, None, None], g2.shape).copy(), dtype=td, device="cuda")
    zeu = torch.zeros(g2.Nx * g2.Ny, dtype=td, device="cuda")
    obgc.euphotic_depth(g2, PAR, zeu, surface_PAR=100.0)
    torch.cuda.synchronize()
    np.testing.assert_allclose(zeu.cpu().numpy(), -10 * np.log(1000), atol=1e-2)


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_mode_i_tendencies_all_configurations(dtype):
    torch = cuda()
    td = torch.float64 if dtype == "f64" else torch.float32
    g = obgc.RectilinearGrid((33, 3, 2), (1.0, 1.0, 2.0))
    lib = A.load()
    rng = np.random.default_rng(5)
    worst = 0.0
    for _, p in ALL:
        names = O.required_tracers(p)
        vals = np.zeros((g.N, A.NUM_NAMED))
        for c in range(g.N):
            for k, v in initial_values(p, rng).items():
                vals[c, A.NAME_INDEX[k]] = v
        PAR = rng.uniform(0, 250, g.N)
        fields = [torch.as_tensor(vals[:, n].copy(), dtype=td, device="cuda") for n in range(A.NUM_NAMED)]
        Gs = [torch.full((g.N,), 12345.0, dtype=td, device="cuda") for _ in range(A.NUM_NAMED)]
        fp = (C.c_void_p * A.NUM_NAMED)(*[fields[n].data_ptr() if n in names else None for n in range(A.NUM_NAMED)])
        gp = (C.c_void_p * A.NUM_NAMED)(*[Gs[n].data_ptr() if n in names else None for n in range(A.NUM_NAMED)])
        PARt = torch.as_tensor(PAR, dtype=td, device="cuda")
        A.check(lib.obgc_npd_tendencies(C.byref(p), C.byref(g.c_grid()), A.F64 if dtype == "f64" else A.F32, fp,
                                        PARt.data_ptr(), gp, 0.0, None), "obgc_npd_tendencies")
        torch.cuda.synchronize()
        ref = O.tendencies_array(p, vals.astype(np.float64) if dtype == "f64" else
                                 np.stack([f.double().cpu().numpy() for f in fields], 1), PARt.double().cpu().numpy())
        for n in names:
            # FP64: relative per cell; FP32: relative to the tracer's tendency scale, since
            # tendencies such as Alk = 15/16 NH4' - 17/16 NO3' - ... cancel far below their terms
            worst = max(worst, rel_err(Gs[n].cpu().numpy(), ref[:, n], 1e-9 if dtype == "f64" else 1.0))
    assert worst < (1e-11 if dtype == "f64" else 1e-5), worst


def test_carbon_batch_fp64():
    torch = cuda()
    rng = np.random.default_rng(9)
    n = 5000
    DIC, Alk = rng.uniform(1900, 2300, n), rng.uniform(2150, 2500, n)
    T, S = rng.uniform(-1, 30, n), rng.uniform(30, 38, n)
    cc = obgc.CarbonChemistry()
    dev = lambda a: torch.as_tensor(a, dtype=torch.float64, device="cuda")
    for out, code in (("pHf", A.OUT_PH_FREE), ("pCO2", A.OUT_PCO2), ("fCO2", A.OUT_FCO2), ("Omega", A.OUT_OMEGA)):
        got = cc(dev(DIC), dev(T), dev(S), Alk=dev(Alk), output=out).cpu().numpy()
        ref = O.carbon_chemistry_batch(O.carbon_options(output=code), DIC, Alk, T, S)
        if out == "pHf":
            assert np.max(np.abs(got - ref)) < 1e-10        # the pH statement of the path: 1e-8
        else:
            assert rel_err(got, ref) < 1e-10


def test_carbon_doctest_digits_on_gpu():
    torch = cuda()
    from test_oracle_carbon import doctest_density
    cc = obgc.CarbonChemistry(density=doctest_density())
    one = lambda x: torch.tensor([x], dtype=torch.float64, device="cuda")
    assert cc(one(2000.0), one(10.0), one(35.0), Alk=one(2000.0)).item() == pytest.approx(1308.1474527899106, rel=1e-13)
    assert cc(one(2000.0), one(10.0), one(35.0), Alk=one(2000.0), output="pHf").item() == pytest.approx(7.502532746463654, rel=1e-14)
    assert cc(one(2000.0), one(10.0), one(35.0), pH=one(7.5)).item() == pytest.approx(1315.7136384737507, rel=1e-13)


def test_carbon_warm_start_and_f32_inputs():
    torch = cuda()
    rng = np.random.default_rng(4)
    n = 2048
    DIC = torch.as_tensor(rng.uniform(2000, 2200, n), dtype=torch.float32, device="cuda")
    Alk = torch.as_tensor(rng.uniform(2300, 2450, n), dtype=torch.float32, device="cuda")
    T = torch.as_tensor(rng.uniform(5, 25, n), dtype=torch.float32, device="cuda")
    S = torch.full((n,), 35.0, dtype=torch.float32, device="cuda")
    cc = obgc.CarbonChemistry()
    H = torch.zeros(n, dtype=torch.float64, device="cuda")
    it1 = torch.zeros(n, dtype=torch.int32, device="cuda")
    it2 = torch.zeros(n, dtype=torch.int32, device="cuda")
    ph1 = cc(DIC, T, S, Alk=Alk, output="pHf", H=H, iters=it1)
    ph2 = cc(DIC, T, S, Alk=Alk, output="pHf", H=H, warm_start=True, iters=it2)
    torch.cuda.synchronize()
    assert torch.max(torch.abs(ph1 - ph2)).item() < 1e-12
    assert it2.float().mean().item() < it1.float().mean().item()
    ref = O.carbon_chemistry_batch(O.carbon_options(output=A.OUT_PH_FREE), DIC.double().cpu().numpy(),
                                   Alk.double().cpu().numpy(), T.double().cpu().numpy(), S.double().cpu().numpy())
    assert np.max(np.abs(ph1.cpu().numpy() - ref)) < 1e-10


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 1e-3)])
def test_box_models_match_oracle(precision, tol):
    torch = cuda()
    rng = np.random.default_rng(6)
    par_fn = lambda t: (60 * (1 - math.cos((t + 15 * 86400) * 2 * math.pi / (365 * 86400))) + 2) * math.exp(-2)
    for base in ("LOBSTER", "NPZD"):
        g = obgc.BoxModelGrid()
        light = obgc.PrescribedPhotosyntheticallyActiveRadiation(par_fn)
        bgc = obgc.LOBSTER(g, light_attenuation=light, carbonate_system=obgc.CarbonateSystem()) if base == "LOBSTER" \
            else obgc.NPZD(g, light_attenuation=light)
        n = 64
        box = obgc.BoxModel(bgc, n_models=n, precision=precision)
        init = {"NO3": 10.0, "NH4": 0.1, "P": 0.1, "Z": 0.01, "DIC": 2200.0, "Alk": 2400.0} if base == "LOBSTER" \
            else {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 12.0}
        for k, v in init.items():
            box.set(**{k: torch.as_tensor(v * rng.uniform(0.8, 1.2, n), dtype=torch.float64, device="cuda")})
        start = box.state.cpu().numpy().copy()
        dt, nsteps = 1200.0, 200
        box.run(dt, nsteps)
        torch.cuda.synchronize()
        got = box.state.cpu().numpy()
        stages = np.array([par_fn(dt * (s + c)) for s in range(nsteps) for c in (0, 8 / 15, 2 / 3)])
        for m in range(0, n, 7):
            v = dict(enumerate(start[m]))
            ref = O.box_run(bgc.params, v, dt, nsteps, PAR_stages=stages)
            assert rel_err(got[m], ref, 1e-9) < tol


def test_box_record_and_per_model_params():
    torch = cuda()
    g = obgc.BoxModelGrid()
    bgc = obgc.NPZD(g, light_attenuation=obgc.PrescribedPhotosyntheticallyActiveRadiation(30.0))
    n = 8
    ps = []
    for q in range(n):
        p = bgc.params.copy()
        p.phytoplankton_maximum_growth_rate *= 1 + 0.1 * q
        ps.append(p)
    box = obgc.BoxModel(bgc, n_models=n, params_per_model=ps)
    box.set(N=10.0, P=0.1, Z=0.01, T=12.0)
    rec = box.run(1200.0, 100, record_every=20)
    torch.cuda.synchronize()
    assert rec.shape == (5, n, A.NUM_NAMED)
    for q in (0, 5):
        ref = O.box_run(ps[q], {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 12.0}, 1200.0, 100, PAR_const=30.0)
        assert rel_err(box.state[q].cpu().numpy(), ref, 1e-9) < 1e-12
        assert rel_err(rec[-1, q].cpu().numpy(), ref, 1e-9) < 1e-12
    assert not np.allclose(box.state[0].cpu().numpy(), box.state[5].cpu().numpy())


@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_mode_i_zero_state_all_configurations(dtype):
    torch = cuda()
    td = torch.float64 if dtype == "f64" else torch.float32
    g = obgc.RectilinearGrid((8, 2, 2), (1.0, 1.0, 2.0))
    lib = A.load()
    zero = torch.zeros(g.N, dtype=td, device="cuda")
    PAR = torch.full((g.N,), 100.0, dtype=td, device="cuda")
    for _, p in ALL:
        names = O.required_tracers(p)
        Gs = [torch.full((g.N,), 7.0, dtype=td, device="cuda") for _ in range(A.NUM_NAMED)]
        fp = (C.c_void_p * A.NUM_NAMED)(*[zero.data_ptr() if n in names else None for n in range(A.NUM_NAMED)])
        gp = (C.c_void_p * A.NUM_NAMED)(*[Gs[n].data_ptr() if n in names else None for n in range(A.NUM_NAMED)])
        A.check(lib.obgc_npd_tendencies(C.byref(p), C.byref(g.c_grid()), A.F64 if dtype == "f64" else A.F32, fp,
                                        PAR.data_ptr(), gp, 0.0, None), "obgc_npd_tendencies")
        torch.cuda.synchronize()
        for n in names:
            assert torch.count_nonzero(Gs[n]).item() == 0


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("f32", 1e-3)])
def test_box_model_forcing_and_prescribed_tracers_match_oracle(precision, tol):
    # BoxModel(; forcing, prescribed_tracers) (boxmodel.jl:65-87): NPZD with a seasonal temperature
    # prescribed as T(t) (it drives the Q10 growth) and a nutrient supply forcing N
    torch = cuda()
    g = obgc.BoxModelGrid()
    bgc = obgc.NPZD(g, light_attenuation=obgc.PrescribedPhotosyntheticallyActiveRadiation(40.0))
    temp = lambda t: 10 + 6 * math.sin(2 * math.pi * t / (20 * 86400))       # noqa: E731
    supply = lambda t: 2e-6 * (1 + math.cos(2 * math.pi * t / (5 * 86400)))  # noqa: E731
    n = 16
    box = obgc.BoxModel(bgc, n_models=n, precision=precision, prescribed_tracers={"T": temp}, forcing={"N": supply})
    box.set(N=10.0, P=0.1, Z=0.01, T=0.0)
    dt, nsteps = 1200.0, 300
    for _ in range(2):                      # two calls: the series continue from the model's clock
        box.run(dt, nsteps // 2)
    torch.cuda.synchronize()
    got = box.state.cpu().numpy()
    times = np.array([dt * (s + c) for s in range(nsteps + 1) for c in (0, 8 / 15, 2 / 3)])
    ref = O.box_run_drivers(bgc.params, {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 0.0}, dt, nsteps, PAR_const=40.0,
                            prescribed={"T": [temp(t) for t in times[:3 * nsteps + 1]]},
                            forcing={"N": [supply(t) for t in times[:3 * nsteps]]})
    for m in (0, n - 1):
        assert rel_err(got[m], ref, 1e-9) < tol
    assert got[0, A.NAME_INDEX["T"]] == pytest.approx(temp(dt * nsteps), rel=1e-6)
    # the forcing and the prescribed temperature changed the outcome
    plain = O.box_run(bgc.params, {"N": 10.0, "P": 0.1, "Z": 0.01, "T": 0.0}, dt, nsteps, PAR_const=40.0)
    assert abs(plain[A.NAME_INDEX["P"]] - ref[A.NAME_INDEX["P"]]) > 1e-3 * abs(ref[A.NAME_INDEX["P"]])
