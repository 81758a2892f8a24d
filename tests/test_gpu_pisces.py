"""PISCES on the GPU against the oracle: all 24 tendencies of every cell of a 3-D grid (FP64 and
FP32) with 2-D, 3-D, constant and computed auxiliary inputs; mixed-layer means; calcite saturation
with the pressure of the cell's depth."""
import numpy as np
import pytest

import obgc
import oracle as O
from obgc import _abi as A
from obgc import pisces as PI
from gpuhelp import cuda
from test_oracle_pisces import INITIAL

pytestmark = pytest.mark.gpu


def setup(dtype, shape=(7, 5, 12), extent=(700.0, 500.0, 240.0), seed=0):
    torch = cuda()
    g = obgc.RectilinearGrid(shape, extent, dtype=dtype)
    td = torch.float32 if dtype == "f32" else torch.float64
    rng = np.random.default_rng(seed)
    host = {}
    for n in A.PISCES_ASCII:
        base = INITIAL.get(n, 0.0)
        host[n] = base * np.exp(rng.normal(0, 0.4, g.shape)) if n not in ("T", "S") else np.full(g.shape, base)
    host["T"] = 4 + 10 * np.exp(g.znodes()[:, None, None] / 100) * np.ones(g.shape)
    zmxl = -rng.uniform(20, 120, (g.Ny, g.Nx))
    zeu = -rng.uniform(30, 150, (g.Ny, g.Nx))
    par = lambda s: 100 * np.exp(g.znodes()[:, None, None] / s) * np.ones(g.shape)   # noqa: E731
    aux_host = dict(zmxl=zmxl, zeu=zeu, Si_clim=7.5, Omega=rng.uniform(0.5, 3, g.shape), kappa=rng.uniform(0.2, 2, (g.Ny, g.Nx)),
                    mixed_layer_PAR=rng.uniform(10, 150, (g.Ny, g.Nx)), PAR=3 * par(30), PAR1=par(20), PAR2=par(30),
                    PAR3=par(10))
    dev = {n: torch.as_tensor(host[n], dtype=td, device="cuda").contiguous() for n in A.PISCES_ASCII}
    aux_dev = {k: (v if isinstance(v, float) else torch.as_tensor(v, dtype=td, device="cuda").contiguous())
               for k, v in aux_host.items()}
    aux_dev["wPOC"] = "auto"
    aux_dev["wGOC"] = "auto"
    return torch, g, host, aux_host, dev, aux_dev


def oracle_cells(p, g, host, aux_host, t):
    zc = g.znodes()
    dz = g.Lz / g.Nz
    poc_faces = np.array([-(p.poc_sinking_speed) if f < g.Nz else 0.0 for f in range(g.Nz + 1)])
    out = np.zeros((24,) + g.shape)
    for j in range(g.Ny):
        for i in range(g.Nx):
            zm, ze = aux_host["zmxl"][j, i], aux_host["zeu"][j, i]
            goc_faces = O.goc_speed(p, zc, zm, ze)
            for k in range(g.Nz):
                v = [host[n][k, j, i] for n in A.PISCES_ASCII]
                a = [zm, ze, 7.5, aux_host["Omega"][k, j, i], aux_host["kappa"][j, i], aux_host["mixed_layer_PAR"][j, i],
                     0.5 * (poc_faces[k] + poc_faces[k + 1]), 0.5 * (goc_faces[k] + goc_faces[k + 1]),
                     aux_host["PAR"][k, j, i], aux_host["PAR1"][k, j, i], aux_host["PAR2"][k, j, i], aux_host["PAR3"][k, j, i]]
                out[:, k, j, i] = O.pisces_tendencies(p, v, a, zc[k], t)
    assert abs(zc[1] - zc[0] - dz) < 1e-9
    return out


@pytest.mark.parametrize("dtype,tol", [("f64", 1e-10), ("f32", 2e-3)])
def test_pisces_tendencies_match_oracle(dtype, tol):
    torch, g, host, aux_host, dev, aux_dev = setup(dtype)
    bgc = PI.PISCES(g)
    G = {n: torch.zeros_like(dev[n]) for n in A.PISCES_ASCII[:24]}
    t = 3.7e6
    PI.pisces_tendencies(bgc, g, dev, aux_dev, G, t=t)
    torch.cuda.synchronize()
    ref = oracle_cells(O.pisces_defaults(), g, {n: dev[n].double().cpu().numpy() for n in A.PISCES_ASCII}, aux_host, t)
    worst = {}
    for q, n in enumerate(A.PISCES_ASCII[:24]):
        got = G[n].double().cpu().numpy()
        # error relative to the tracer's largest tendency term: the budget terms cancel in several
        # tracers, so a cell's net tendency can be far below the rounding of its terms in FP32
        scale = np.max(np.abs(ref[q]))
        worst[n] = float(np.max(np.abs(got - ref[q])) / max(scale, 1e-300))
    assert max(worst.values()) < tol, worst


def test_mixed_layer_mean_and_calcite_saturation():
    torch, g, host, aux_host, dev, aux_dev = setup("f64")
    out = torch.zeros((g.Ny, g.Nx), dtype=torch.float64, device="cuda")
    PI.mixed_layer_mean(g, dev["T"], aux_dev["zmxl"], out)
    zf = -g.Lz + g.Lz / g.Nz * np.arange(g.Nz + 1)
    T = host["T"]
    for j in range(g.Ny):
        for i in range(g.Nx):
            assert out[j, i].item() == pytest.approx(O.mixed_layer_mean(zf, T[:, j, i], aux_host["zmxl"][j, i]), rel=1e-13)
    om = torch.zeros(g.shape, dtype=torch.float64, device="cuda")
    PI.calcite_saturation(g, dev["DIC"], dev["Alk"], dev["T"], dev["S"], dev["Si"], om)
    zc = g.znodes()
    for (k, j, i) in [(0, 0, 0), (5, 2, 3), (11, 4, 6)]:
        P = abs(zc[k]) * 9.80665 * 1026 / 100000
        ref = O.carbon_chemistry(host["DIC"][k, j, i], host["T"][k, j, i], host["S"][k, j, i], Alk=host["Alk"][k, j, i],
                                 P=P, silicate=host["Si"][k, j, i], output=A.OUT_OMEGA)
        assert om[k, j, i].item() == pytest.approx(ref, rel=1e-10)
