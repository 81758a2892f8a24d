"""Seeded synthetic inputs with the shapes and value distributions of the reference's configurations
(no datasets exist for them): LOBSTER 3-D initial conditions and a divergence-free velocity from a
random streamfunction.
"""
import numpy as np


def random_streamfunction_velocity(grid, rms=0.1, seed=0, modes=6, device="cuda", dtype=None):
    """u = -dpsi/dy, v = dpsi/dx from a seeded random psi at (Face, Face, Center), scaled to the
    given RMS speed; w = 0.  The differences are taken on the grid, so the discrete divergence
    (u[i+1]-u[i])/dx + (v[j+1]-v[j])/dy vanishes to rounding."""
    import torch
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz = grid.Nx, grid.Ny, grid.Nz
    x = np.arange(Nx) / Nx
    y = np.arange(Ny) / Ny
    zc = np.linspace(0, 1, Nz)
    psi = np.zeros((Nz, Ny, Nx))
    for _ in range(modes):
        kx, ky = rng.integers(1, 5, size=2)
        ph = rng.uniform(0, 2 * np.pi, size=2)
        a = rng.normal()
        vert = 1 + 0.5 * np.cos(np.pi * zc * rng.integers(1, 3) + rng.uniform(0, 2 * np.pi))
        psi += a * vert[:, None, None] * np.cos(2 * np.pi * kx * x[None, None, :] + ph[0]) * \
               np.cos(2 * np.pi * ky * y[None, :, None] + ph[1])
    dx, dy = grid.Lx / Nx, grid.Ly / Ny
    u = -(np.roll(psi, -1, axis=1) - psi) / dy          # at (Face, Center): psi(i, j+1) - psi(i, j)
    v = (np.roll(psi, -1, axis=2) - psi) / dx           # at (Center, Face): psi(i+1, j) - psi(i, j)
    speed = np.sqrt(np.mean(u ** 2 + v ** 2))
    u *= rms / speed
    v *= rms / speed
    dt = dtype or torch.float64
    return (torch.as_tensor(u, dtype=dt, device=device), torch.as_tensor(v, dtype=dt, device=device), None)


def correlated_normal(shape, rng, length=(1.0, 2.0, 2.0)):
    """Standard-normal field (zero mean, unit variance per cell) with Gaussian spatial correlation
    of the given length in cells along (z, y, x), periodic in every direction."""
    white = rng.standard_normal(shape)
    spec = np.fft.rfftn(white)
    kz = np.fft.fftfreq(shape[0])[:, None, None]
    ky = np.fft.fftfreq(shape[1])[None, :, None]
    kx = np.fft.rfftfreq(shape[2])[None, None, :]
    filt = np.exp(-2 * np.pi ** 2 * ((kz * length[0]) ** 2 + (ky * length[1]) ** 2 + (kx * length[2]) ** 2))
    f = np.fft.irfftn(spec * filt, s=shape)
    f -= f.mean()
    return f / f.std()


def _uniform(g, lo, hi):
    """Map a standard-normal field to U(lo, hi) through the normal CDF."""
    return lo + (hi - lo) * 0.5 * (1 + _erf(g / np.sqrt(2)))


def _erf(x):
    # Abramowitz & Stegun 7.1.26 (|error| < 1.5e-7): only shapes a uniform marginal
    s = np.sign(x)
    a = np.abs(x)
    t = 1 / (1 + 0.3275911 * a)
    y = 1 - (((((1.061405429 * t - 1.453152027) * t) + 1.421413741) * t - 0.284496736) * t + 0.254829592) * t * np.exp(-a * a)
    return s * y


def lobster_initial_conditions(grid, seed=0, correlated=True):
    """NO3 ~ U(5,15); P, Z ~ LogNormal(log 0.1, 0.5); DIC ~ U(2100,2250); Alk ~ U(2300,2450);
    T = 12 - 0.01 z; S = 35; NH4, sPOM, bPOM, DOM = 0.  With `correlated`, each field keeps that
    marginal distribution but is spatially correlated over ~2 cells (white noise at the grid scale
    drives WENO undershoots, and a negative P makes the (P R/r)^e of the light model undefined)."""
    rng = np.random.default_rng(seed)
    shp = grid.shape
    z = grid.znodes()[:, None, None] * np.ones(shp)
    if correlated:
        n = lambda: correlated_normal(shp, rng)
        return {
            "NO3": _uniform(n(), 5, 15), "NH4": 0.0,
            "P": np.exp(np.log(0.1) + 0.5 * n()), "Z": np.exp(np.log(0.1) + 0.5 * n()),
            "sPOM": 0.0, "bPOM": 0.0, "DOM": 0.0,
            "DIC": _uniform(n(), 2100, 2250), "Alk": _uniform(n(), 2300, 2450),
            "T": 12 - 0.01 * z, "S": 35.0,
        }
    return {
        "NO3": rng.uniform(5, 15, shp), "NH4": 0.0,
        "P": rng.lognormal(np.log(0.1), 0.5, shp), "Z": rng.lognormal(np.log(0.1), 0.5, shp),
        "sPOM": 0.0, "bPOM": 0.0, "DOM": 0.0,
        "DIC": rng.uniform(2100, 2250, shp), "Alk": rng.uniform(2300, 2450, shp),
        "T": 12 - 0.01 * z, "S": 35.0,
    }


# PISCES_INITIAL_VALUES of the reference's PISCES tests (test/test_PISCES.jl:8-16): the surface
# value of each profile below
PISCES_SURFACE_VALUES = dict(P=0.5, PChl=0.02, PFe=0.005, D=0.1, DChl=0.004, DFe=0.001, DSi=0.01, Z=0.1, M=0.7,
                             DOC=2.1, POC=7.8, SFe=0.206, GOC=38, BFe=1.1, PSi=0.1, CaCO3=1e-10, NO3=2.3, NH4=0.9,
                             PO4=0.6, Fe=0.13, Si=8.5, DIC=2205, Alk=2566, O2=317, T=10, S=35)


def pisces_initial_conditions(grid, seed=0, noise=0.05):
    """Depth profiles for the 26 PISCES tracers with spatially correlated lognormal noise of the
    given relative size on every tracer but T and S: living and particulate pools decay below the
    surface over 100 m to 5% of their surface value, nutrients grow fourfold over ~250 m, DIC and
    Alk rise by 100 and 20 umol/kg, O2 falls to 60% and T from 18 to 4 C over ~200 m."""
    rng = np.random.default_rng(seed)
    shp = grid.shape
    z = grid.znodes()[:, None, None] * np.ones(shp)
    v = PISCES_SURFACE_VALUES
    surf = 0.05 + 0.95 * np.exp(z / 100)
    deep = 1 + 3 * (1 - np.exp(z / 250))
    out = {}
    for n in ("P", "PChl", "PFe", "D", "DChl", "DFe", "DSi", "Z", "M", "DOC", "POC", "SFe", "GOC", "BFe", "PSi", "CaCO3"):
        out[n] = v[n] * surf
    for n in ("NO3", "PO4", "Si", "Fe"):
        out[n] = v[n] * deep
    out["NH4"] = v["NH4"] * (0.2 + 0.8 * np.exp(z / 100))
    out["DIC"] = v["DIC"] + 100 * (1 - np.exp(z / 300))
    out["Alk"] = v["Alk"] + 20 * (1 - np.exp(z / 300))
    out["O2"] = v["O2"] * (0.6 + 0.4 * np.exp(z / 200))
    for n in list(out):
        out[n] = out[n] * np.exp(noise * correlated_normal(shp, rng))
    out["T"] = 4 + 14 * np.exp(z / 200)
    out["S"] = np.full(shp, 35.0)
    return out


def npzd_front_initial_conditions(grid):
    """README.md:46-52 (the buoyancy-front example): N = 2.5 - 2 tanh((x - 7000 + 4z)/500),
    T = 9 + 0.05 tanh(...), P = Z = 0.03 above -50 m and 0.01 below, D = 0."""
    x = (np.arange(grid.Nx) + 0.5) * grid.Lx / grid.Nx
    z = grid.znodes()
    X = x[None, None, :] * np.ones(grid.shape)
    Zc = z[:, None, None] * np.ones(grid.shape)
    front = np.tanh((X - 7000 + 4 * Zc) / 500)
    PZ = np.where(Zc > -50, 0.03, 0.01)
    return {"N": 2.5 - 2 * front, "T": 9 + 0.05 * front, "P": PZ, "Z": PZ.copy(), "D": 0.0}


def mixed_layer_diffusivity(Nz, dz, mld, kappa_mixed=1e-2, kappa_deep=1e-4, width=10.0):
    """Face diffusivities (bottom face first) of the reference's column example profile
    kappa(z) = kappa_mixed (1 + tanh((z + mld) / width)) / 2 + kappa_deep (examples/column.jl:34)."""
    zf = -Nz * dz + dz * np.arange(Nz + 1)
    return kappa_mixed * (1 + np.tanh((zf + mld) / width)) / 2 + kappa_deep


def npzd_column_ensemble(n, seed=0, levels=(16, 256), dz=2.0, dt=600.0, nsteps=1440):
    """Seeded uneven NPZD columns: Nz ~ U{levels}, dz = 2 m, maximum phytoplankton growth
    ~ lognormal(log 1.5e-5 s^-1, 0.3), mixed-layer depth ~ U(20, 200) m setting the diffusivity
    1e-4 .. 1e-2 m^2/s (mixed_layer_diffusivity), surface PAR ~ U(50, 300) W/m^2.  Initial profiles
    follow the NPZD front example's values: N rising from 2.5 at the surface to 10 at depth,
    P = Z = 0.03 in the mixed layer and 0.01 below, D = 0, T = 12 + 0.01 z.  Each column is a dict
    with init [N, P, Z, T, D] x Nz (bottom first), kappa, dz, dt, nsteps, surface_PAR, mu0."""
    rng = np.random.default_rng(seed)
    cols = []
    for _ in range(n):
        Nz = int(rng.integers(levels[0], levels[1] + 1))
        mld = rng.uniform(20, 200)
        z = -Nz * dz + dz * (np.arange(Nz) + 0.5)
        inside = z > -mld
        N = 2.5 + 7.5 * (1 - np.exp(z / 150.0))
        P = np.where(inside, 0.03, 0.01)
        init = np.stack([N, P, P.copy(), 12 + 0.01 * z, np.zeros(Nz)])
        cols.append(dict(init=init, kappa=mixed_layer_diffusivity(Nz, dz, mld), dz=dz, dt=dt, nsteps=nsteps,
                         surface_PAR=rng.uniform(50, 300), mu0=float(np.exp(rng.normal(np.log(1.5e-5), 0.3)))))
    return cols


def lobster_column_request(rng, levels=(8, 512), days=(1, 30), dts=(300.0, 1800.0), pulse=(0.0, 500.0),
                           w_max=0.0023148148148148147):
    """One column-run request of the alkalinity-addition scenario service: LOBSTER with carbonates,
    Nz log-uniform in `levels`, duration U(days), dt U(dts), an alkalinity pulse U(pulse) added at a
    random level and step.  The level thickness is U(2, 10) m but at least 1.5 w_max dt, so the
    explicit sinking of large particles stays below CFL 0.7.  Values: NO3 ~ U(5, 15), NH4 0.05,
    P, Z ~ lognormal(log 0.1, 0.5) in the mixed layer (a tenth below), sPOM = bPOM = DOM = 0.01,
    DIC ~ U(2100, 2250), Alk ~ U(2300, 2450); surface T ~ U(2, 28) degC and S ~ U(33, 37) for the
    CO2 gas exchange."""
    Nz = int(np.exp(rng.uniform(np.log(levels[0]), np.log(levels[1] + 1))))
    Nz = max(levels[0], min(levels[1], Nz))
    dt = float(rng.uniform(*dts))
    dz = max(float(rng.uniform(2, 10)), 1.5 * w_max * dt)
    nsteps = max(1, int(round(rng.uniform(*days) * 86400.0 / dt)))
    mld = rng.uniform(20, 200)
    z = -Nz * dz + dz * (np.arange(Nz) + 0.5)
    inside = z > -mld
    scale = np.where(inside, 1.0, 0.1)
    P = np.exp(rng.normal(np.log(0.1), 0.5, Nz)) * scale
    Zp = np.exp(rng.normal(np.log(0.1), 0.5, Nz)) * scale
    init = np.stack([np.full(Nz, rng.uniform(5, 15)), np.full(Nz, 0.05), P, Zp, np.full(Nz, 0.01), np.full(Nz, 0.01),
                     np.full(Nz, 0.01), np.full(Nz, rng.uniform(2100, 2250)), np.full(Nz, rng.uniform(2300, 2450))])
    return dict(init=init, kappa=mixed_layer_diffusivity(Nz, dz, mld), dz=dz, dt=dt, nsteps=nsteps,
                surface_PAR=float(rng.uniform(50, 300)), mu0=0.0, pulse_step=int(rng.integers(0, nsteps)),
                pulse_k=int(rng.integers(0, Nz)), pulse_amount=float(rng.uniform(*pulse)),
                T=float(rng.uniform(2, 28)), S=float(rng.uniform(33, 37)))
