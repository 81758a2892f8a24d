"""The fused substep with TMA-staged tiles (the MODE 2 kernel, every tile of a level copied with
one tensor copy per tracer): a call copies the bound arrays into padded copy 1 with their periodic
images (pad_copy_kernel), then its stages run padded copy 1 -> padded copy 0 -> padded copy 1 ...
-> bound arrays; when no tile needs the periodic wrap and the bound arrays' layout allows tensor maps,
the first stage copies its tiles from the bound arrays directly.  The arithmetic per cell is the
same as with cp.async staging, so the two agree bit for bit, on grids whose sizes are not multiples
of the 32 x 8 tile (tiles hang over the padded arrays' edges), with walls as well as periodic
directions, and with a row pitch that allows no tensor map of the bound arrays; and both agree with
the oracle.  The mixed path (FP64 state, FP32 arithmetic) stages its tiles the same way from FP32
padded copies (the copy rounds the state, each stage but the last writes the next copy) and
updates its FP64 state in place; it equals its own cp.async staging bit for bit too."""
import numpy as np
import pytest

import obgc
import oracle as O
from gpuhelp import cuda, rel_err

pytestmark = pytest.mark.gpu


def run(shape, topology, staging, nsteps=3, graph=False, seed=2, precision="f32", tiling=None):
    torch = cuda()
    L = (shape[0] * 195.3125, shape[1] * 195.3125, shape[2] * 7.8125)
    f32 = precision == "f32"
    g = obgc.RectilinearGrid(shape, L, topology, dtype="f32" if f32 else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=seed, dtype=torch.float32 if f32 else torch.float64)
    m = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None), precision=precision)
    m.set_staging(staging)
    if tiling is not None:
        m.set_tiling(tiling)
    obgc.set_(m, **obgc.lobster_initial_conditions(g, seed=seed + 1))
    s0 = m.state_array().double().cpu().numpy()
    obgc.time_step(m, 300.0, nsteps=nsteps, graph=graph)
    torch.cuda.synchronize()
    return g, bgc, (u, v), m, s0, m.state_array().double().cpu().numpy()


@pytest.mark.parametrize("shape,topology", [
    ((40, 20, 12), ("Periodic", "Periodic", "Bounded")),     # tiles overhang in x and y
    ((64, 16, 9), ("Periodic", "Periodic", "Bounded")),
    ((36, 24, 8), ("Bounded", "Periodic", "Bounded")),
    ((32, 19, 10), ("Periodic", "Bounded", "Bounded")),
    ((96, 32, 8), ("Periodic", "Periodic", "Bounded")),     # wrapping and wrap-free tiles
    ((100, 28, 6), ("Bounded", "Periodic", "Bounded")),
    ((37, 20, 8), ("Periodic", "Periodic", "Bounded")),     # 148-byte rows: no tensor map of the bound arrays
    ((64, 32, 8), ("Bounded", "Bounded", "Bounded")),       # no tile wraps: no copy, the bound arrays' tensor maps
])
def test_tma_staging_equals_cp_async_staging(shape, topology):
    _, _, _, m1, _, tma = run(shape, topology, staging=1)
    assert m1.staging() == (True, True)
    _, _, _, m0, _, ref = run(shape, topology, staging=0)
    assert m0.staging() == (True, False)
    assert np.array_equal(tma, ref), max(rel_err(tma[q], ref[q]) for q in range(tma.shape[0]))
    assert m1.step_status() == (0, 0)


def test_tma_staging_matches_oracle_and_graph_replay():
    shape, topo = (48, 24, 16), ("Periodic", "Periodic", "Bounded")
    g, bgc, (u, v), m, s0, got = run(shape, topo, staging=1, nsteps=4)
    mo = O.model3d(bgc.params, g.c_grid(), m.tracer_names)
    ref = np.ascontiguousarray(s0.copy())
    O.step3d(mo, ref, u=u.double().cpu().numpy().ravel().copy(), v=v.double().cpu().numpy().ravel().copy(),
             t=0.0, dt=300.0, nsteps=4)
    assert max(rel_err(got[q], ref[q]) for q in range(got.shape[0])) < 5e-5
    # the same four steps replayed from a CUDA graph
    _, _, _, mg, _, gg = run(shape, topo, staging=1, nsteps=4, graph=True)
    assert mg.staging() == (True, True)
    assert np.array_equal(gg, got)


@pytest.mark.parametrize("shape", [(6, 16, 8), (32, 5, 8)])
def test_periodic_grids_narrower_than_two_halos_keep_cp_async(shape):
    # one periodic image per cell and side fills the padded halos only when a periodic direction has
    # at least 8 (x) or 6 (y) cells: narrower grids stay on cp.async staging, and agree with it
    topo = ("Periodic", "Periodic", "Bounded")
    _, _, _, m1, _, got = run(shape, topo, staging=1)
    assert m1.staging() == (True, False)
    _, _, _, m0, _, ref = run(shape, topo, staging=0)
    assert np.array_equal(got, ref)


def test_configurations_outside_the_lean_kernel_keep_cp_async():
    torch = cuda()
    g = obgc.RectilinearGrid((32, 16, 8), (6250.0, 3125.0, 62.5), dtype="f32")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem(), scale_negatives=True)
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=1, dtype=torch.float32)
    m = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None), precision="f32")
    m.set_staging(1)
    obgc.set_(m, **obgc.lobster_initial_conditions(g, seed=2))
    obgc.time_step(m, 300.0, nsteps=1)
    assert m.staging() == (True, False)          # the fused modifier needs the extended kernel
    g64 = obgc.RectilinearGrid((32, 16, 8), (6250.0, 3125.0, 62.5))
    u64, v64, _ = obgc.random_streamfunction_velocity(g64, rms=0.1, seed=1)
    for prec in ("mixed", "f64"):
        mx = obgc.NonhydrostaticModel(g64, biogeochemistry=obgc.LOBSTER(g64, carbonate_system=obgc.CarbonateSystem()),
                                      tracers=("T", "S"), velocities=(u64, v64, None), precision=prec)
        # the padded FP32 copies exist for FP32 arithmetic only
        assert mx.staging() == ((True, False) if prec == "mixed" else (False, False))


def test_padded_copy_and_stages_in_a_graph():
    # 96 x 32 periodic (some tiles wrap, some do not): the copy into the padded set and the stages,
    # captured into a CUDA graph, give the same state as eager calls
    shape, topo = (96, 32, 8), ("Periodic", "Periodic", "Bounded")
    _, _, _, me, _, eager = run(shape, topo, staging=1, nsteps=2)
    _, _, _, mg, _, graph = run(shape, topo, staging=1, nsteps=2, graph=True)
    assert mg.staging() == (True, True)
    assert np.array_equal(graph, eager)
    # one step per call, as an ensemble host drives it
    _, _, _, m1, _, one = run(shape, topo, staging=1, nsteps=1)
    _, _, _, m0, _, ref = run(shape, topo, staging=0, nsteps=1)
    assert np.array_equal(one, ref)


def test_ensemble_members_through_host_copies_equal_eager_steps():
    # two members stepped in turn from CUDA graphs, each step's state copied in from pinned host
    # memory and back (the bench's end-to-end pipeline), equal one member stepped eagerly
    torch = cuda()
    shape, topo = (96, 32, 8), ("Periodic", "Periodic", "Bounded")
    _, _, _, _, _, ref = run(shape, topo, staging=1, nsteps=3)
    L = (shape[0] * 195.3125, shape[1] * 195.3125, shape[2] * 7.8125)
    g = obgc.RectilinearGrid(shape, L, topo, dtype="f32")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=2, dtype=torch.float32)
    members = []
    for q in range(2):
        m = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None), precision="f32")
        obgc.set_(m, **obgc.lobster_initial_conditions(g, seed=3))
        host = {n: m.tracers[n].cpu().pin_memory() for n in m.tracer_names}
        members.append((m, host))
    for _ in range(3):
        for m, host in members:
            for n in m.tracer_names:
                m.tracers[n].copy_(host[n], non_blocking=True)
            obgc.time_step(m, 300.0, nsteps=1, graph=True)
            for n in m.tracer_names:
                host[n].copy_(m.tracers[n], non_blocking=True)
    torch.cuda.synchronize()
    for m, host in members:
        got = np.stack([host[n].double().numpy() for n in m.tracer_names])
        assert np.array_equal(got, ref)


@pytest.mark.parametrize("shape,topology", [
    ((40, 20, 12), ("Periodic", "Periodic", "Bounded")),
    ((96, 32, 8), ("Periodic", "Periodic", "Bounded")),
    ((36, 24, 8), ("Bounded", "Periodic", "Bounded")),
    ((64, 32, 8), ("Bounded", "Bounded", "Bounded")),       # no tile wraps: still the rounding copy
])
def test_mixed_tma_staging_equals_cp_async_staging(shape, topology):
    _, _, _, m1, _, tma = run(shape, topology, staging=1, precision="mixed")
    assert m1.staging() == (True, True)
    _, _, _, m0, _, ref = run(shape, topology, staging=0, precision="mixed")
    assert m0.staging() == (True, False)
    assert np.array_equal(tma, ref), max(rel_err(tma[q], ref[q]) for q in range(tma.shape[0]))
    assert m1.step_status() == (0, 0)


def test_mixed_tma_staging_matches_oracle_graph_and_one_step_calls():
    shape, topo = (48, 24, 16), ("Periodic", "Periodic", "Bounded")
    g, bgc, (u, v), m, s0, got = run(shape, topo, staging=1, nsteps=4, precision="mixed")
    mo = O.model3d(bgc.params, g.c_grid(), m.tracer_names)
    ref = np.ascontiguousarray(s0.copy())
    O.step3d(mo, ref, u=u.double().cpu().numpy().ravel().copy(), v=v.double().cpu().numpy().ravel().copy(),
             t=0.0, dt=300.0, nsteps=4)
    assert max(rel_err(got[q], ref[q]) for q in range(got.shape[0])) < 1e-5
    _, _, _, mg, _, gg = run(shape, topo, staging=1, nsteps=4, graph=True, precision="mixed")
    assert mg.staging() == (True, True)
    assert np.array_equal(gg, got)
    # four one-step calls (each with its rounding copy) equal one four-step call
    torch = cuda()
    L = (shape[0] * 195.3125, shape[1] * 195.3125, shape[2] * 7.8125)
    g2 = obgc.RectilinearGrid(shape, L, topo, dtype="f64")
    u2, v2, _ = obgc.random_streamfunction_velocity(g2, rms=0.1, seed=2, dtype=torch.float64)
    m2 = obgc.NonhydrostaticModel(g2, biogeochemistry=obgc.LOBSTER(g2, carbonate_system=obgc.CarbonateSystem()),
                                  tracers=("T", "S"), velocities=(u2, v2, None), precision="mixed")
    m2.set_staging(1)
    obgc.set_(m2, **obgc.lobster_initial_conditions(g2, seed=3))
    for _ in range(4):
        obgc.time_step(m2, 300.0, nsteps=1)
    assert np.array_equal(m2.state_array().double().cpu().numpy(), got)


def test_mixed_stages_that_would_read_other_cells_keep_cp_async():
    # one-level segments sum the chlorophyll above each segment in the work items, from other cells of
    # the state that the in-place FP64 update may already have overwritten: cp.async staging
    shape, topo = (40, 20, 12), ("Periodic", "Periodic", "Bounded")
    _, _, _, m1, _, got = run(shape, topo, staging=1, precision="mixed", tiling=1)
    assert m1.staging() == (True, False)
    _, _, _, _, _, ref = run(shape, topo, staging=1, precision="mixed", tiling=4)
    assert np.array_equal(got, ref)
