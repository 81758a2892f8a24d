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
