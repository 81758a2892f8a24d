"""The y slab split on one GPU: the halo pack / unpack kernels against the host layout, and two or
three slabs stepped in lockstep in one process (their exchange a device copy between the slabs'
buffers, where ranks would use NCCL send/recv) against the single-domain fused step and the
oracle.  No kernel waits on another: each slab's stage is its own launch after the copies."""
import ctypes as C

import numpy as np
import pytest

import obgc
from obgc import _abi as A
from gpuhelp import cuda, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", ["f32", "f64"])
def test_halo_pack_and_unpack_match_the_host_layout(dtype):
    torch = cuda()
    tdt = torch.float32 if dtype == "f32" else torch.float64
    g = obgc.RectilinearGrid((10, 11, 4), (1.0, 1.0, 1.0))          # a slab of 5 own rows and 2 x 3 halo rows
    H = 3
    fields = [torch.randn(g.shape, dtype=tdt, device="cuda") for _ in range(3)]
    ptrs = (C.c_void_p * 3)(*[f.data_ptr() for f in fields])
    south = torch.empty((3, g.Nz, H, g.Nx), dtype=tdt, device="cuda")
    north = torch.empty_like(south)
    lib = A.load()
    code = A.F32 if dtype == "f32" else A.F64
    assert lib.obgc_halo_pack(C.byref(g.c_grid()), code, 3, ptrs, H, south.data_ptr(), north.data_ptr(), None) == 0
    torch.cuda.synchronize()
    st = torch.stack(fields)
    assert torch.equal(south, st[:, :, H:2 * H, :])
    assert torch.equal(north, st[:, :, g.Ny - 2 * H:g.Ny - H, :])
    rs, rn = torch.randn_like(south), torch.randn_like(north)
    assert lib.obgc_halo_unpack(C.byref(g.c_grid()), code, 3, ptrs, H, rs.data_ptr(), rn.data_ptr(), None) == 0
    torch.cuda.synchronize()
    st2 = torch.stack(fields)
    assert torch.equal(st2[:, :, :H, :], rs) and torch.equal(st2[:, :, g.Ny - H:, :], rn)
    assert torch.equal(st2[:, :, H:g.Ny - H, :], st[:, :, H:g.Ny - H, :])
    # too few own rows between the halos
    small = obgc.RectilinearGrid((10, 8, 4), (1.0, 1.0, 1.0))
    assert lib.obgc_halo_pack(C.byref(small.c_grid()), code, 3, ptrs, H, south.data_ptr(), north.data_ptr(), None) == 1


def lockstep(slabs, dt, nsteps):
    """The ranks' stages in lockstep; the exchange copies each slab's packed rows into its
    neighbours' receive buffers."""
    for _ in range(nsteps):
        for stage in range(3):
            for s in slabs:
                s.pack_halos()
            for s in slabs:
                d = s.decomposition
                s.recv[0].copy_(slabs[d.south].send[1])     # the southern neighbour's last own rows
                s.recv[1].copy_(slabs[d.north].send[0])     # the northern neighbour's first own rows
            for s in slabs:
                s.run_stage(stage, dt)
    for s in slabs:
        s.sync_fields()


@pytest.mark.parametrize("precision,world", [("f64", 2), ("f32", 2), ("mixed", 3)])
def test_slabs_in_lockstep_equal_the_single_domain_step(precision, world):
    torch = cuda()
    import oracle as O
    shape = (32, 24, 8)
    g = obgc.RectilinearGrid(shape, (6400.0, 4800.0, 80.0), dtype="f32" if precision == "f32" else "f64")
    bgc = obgc.LOBSTER(g, carbonate_system=obgc.CarbonateSystem())
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=5)
    init = obgc.lobster_initial_conditions(g, seed=6)
    dt, nsteps = 300.0, 3

    whole = obgc.NonhydrostaticModel(g, biogeochemistry=bgc, tracers=("T", "S"), velocities=(u, v, None),
                                     precision=precision)
    obgc.set_(whole, **init)
    s0 = whole.state_array().double().cpu().numpy()
    obgc.time_step(whole, dt, nsteps=nsteps)
    ref_gpu = whole.state_array().double().cpu().numpy()

    slabs = [obgc.SlabModel(obgc.SlabDecomposition(g, r, world), bgc, (u, v, None), init, precision=precision)
             for r in range(world)]
    lockstep(slabs, dt, nsteps)
    got = torch.cat([s.own_state() for s in slabs], dim=2).double().cpu().numpy()

    # the same cells through the same kernel arithmetic: the slabs equal the single domain exactly
    assert np.array_equal(got, ref_gpu), max(rel_err(got[q], ref_gpu[q]) for q in range(got.shape[0]))
    # and the oracle (the split does not change the error statement of the path)
    m = O.model3d(bgc.params, g.c_grid(), whole.tracer_names)
    ref = np.ascontiguousarray(s0.copy())
    O.step3d(m, ref, u=u.double().cpu().numpy().ravel().copy(), v=v.double().cpu().numpy().ravel().copy(),
             t=0.0, dt=dt, nsteps=nsteps)
    tol = {"f64": 1e-11, "mixed": 1e-5, "f32": 5e-5}[precision]
    assert max(rel_err(got[q], ref[q]) for q in range(got.shape[0])) < tol


@pytest.mark.parametrize("precision", ["f64", "mixed", "f32"])
def test_pisces_slabs_in_lockstep_equal_the_single_domain_step(precision):
    # configuration 4's model split in two y slabs: the same cells through the same kernels
    torch = cuda()
    g = obgc.RectilinearGrid((16, 12, 10), (16000.0, 12000.0, 500.0), dtype="f32" if precision == "f32" else "f64")
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=4)
    init = obgc.pisces_initial_conditions(g, seed=6)
    dt, nsteps = 600.0, 2
    kw = dict(mixed_layer_depth=-60.0, surface_PAR=100.0)
    whole = obgc.PiscesModel(g, velocities=(u, v), precision=precision, **kw)
    whole.set_(**init)
    whole.time_step(dt, nsteps=nsteps)
    ref = whole.state_array().double().cpu().numpy()
    slabs = [obgc.PiscesSlabModel(obgc.SlabDecomposition(g, r, 2), (u, v), init, precision=precision, **kw)
             for r in range(2)]
    for s in range(nsteps):
        for stage in range(3):
            for sl in slabs:
                sl.pack_halos()
            for sl in slabs:
                d = sl.decomposition
                sl.recv[0].copy_(slabs[d.south].send[1])
                sl.recv[1].copy_(slabs[d.north].send[0])
            for sl in slabs:
                sl.run_stage(stage, dt, finish=(s == nsteps - 1 and stage == 2))
    for sl in slabs:
        sl.sync_fields()
    got = torch.cat([sl.own_state() for sl in slabs], dim=2).double().cpu().numpy()
    assert np.array_equal(got, ref), max(rel_err(got[q], ref[q]) for q in range(got.shape[0]))


def test_pisces_stage_rejects_shared_arrays():
    torch = cuda()
    g = obgc.RectilinearGrid((8, 6, 6), (8000.0, 6000.0, 300.0), dtype="f64")
    m = obgc.PiscesModel(g, precision="f64")
    lib = A.load()
    f = [m.tracers[n] for n in A.PISCES_TRACERS]
    ptrs = (C.c_void_p * 26)(*[x.data_ptr() for x in f])
    assert lib.obgc_pisces_model_substep(m._h, 0.0, 600.0, 0, ptrs, ptrs, 0, None) == 1   # OBGC_ERR_INVALID_ARGUMENT
    assert lib.obgc_pisces_model_substep(m._h, 0.0, 600.0, 3, ptrs, ptrs, 0, None) == 1   # OBGC_ERR_INVALID_ARGUMENT
