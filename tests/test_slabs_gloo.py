"""The y slab split of the 3-D step on CPU ranks (gloo): every rank steps its slab with the
oracle's stage-level RK3 (or_stage3d) and exchanges halo rows through SlabDecomposition.exchange
before each stage; the gathered slabs equal the single-domain oracle bit for bit.  This is the host
logic of the multi-GPU path (rows, neighbours, tags, buffer layout, ping-pong of the stages) with
the oracle standing in for the GPU's stage (the GPU stage itself is checked against the
single-domain GPU step in test_gpu_slabs.py)."""
import os
import socket
import tempfile

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist          # noqa: E402
import torch.multiprocessing as mp        # noqa: E402

SHAPE_BY_WORLD = {2: (16, 16, 8), 3: (12, 18, 6)}
STEPS = 3


def pack_rows(state, d):
    """Host mirror of obgc_halo_pack's buffers: [n][Nz][halo][Nx], south rows then north rows."""
    H, ny = d.halo, d.slab_grid.Ny
    return (np.ascontiguousarray(state[:, :, H:2 * H, :]), np.ascontiguousarray(state[:, :, ny - 2 * H:ny - H, :]))


def unpack_rows(state, d, south, north):
    H, ny = d.halo, d.slab_grid.Ny
    state[:, :, 0:H, :] = south
    state[:, :, ny - H:ny, :] = north


def rank_main(rank, world, port, out_path):
    import conditioning as K
    import oracle as O
    import obgc
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        c = K.LobsterCase(SHAPE_BY_WORLD[world])
        d = obgc.SlabDecomposition(c.grid, rank, world)
        m = O.model3d(c.bgc.params, d.slab_grid.c_grid(), K.NAMES)
        shp = c.grid.shape
        st = np.ascontiguousarray(np.stack([d.scatter(c.state0[q]) for q in range(len(K.NAMES))]))
        u = np.ascontiguousarray(d.scatter(c.u.reshape(shp)).ravel())
        v = np.ascontiguousarray(d.scatter(c.v.reshape(shp)).ravel())
        G, Gm = np.zeros_like(st), np.zeros_like(st)
        rs = torch.empty(d.buffer_shape(len(K.NAMES)), dtype=torch.float64)
        rn = torch.empty_like(rs)
        for n in range(STEPS):
            for stage in range(3):
                ss, sn = pack_rows(st, d)
                d.exchange(torch.from_numpy(ss), torch.from_numpy(sn), rs, rn)
                unpack_rows(st, d, rs.numpy(), rn.numpy())
                O.stage3d(m, st, G, Gm, u=u, v=v, t=n * K.DT, dt=K.DT, stage=stage, threads=1)
                G, Gm = Gm, G
        own = torch.from_numpy(np.ascontiguousarray(st[:, :, d.own(), :]))
        parts = [torch.empty_like(own) for _ in range(world)] if rank == 0 else None
        dist.gather(own, parts, dst=0)
        if rank == 0:
            slabbed = torch.cat(parts, dim=2).numpy()
            ref = c.oracle_run(STEPS, threads=1)
            np.savez(out_path, slabbed=slabbed, ref=ref)
    finally:
        dist.destroy_process_group()


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3])
def test_slabbed_oracle_with_exchanged_halos_equals_single_domain(world):
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "result.npz")
        mp.start_processes(rank_main, args=(world, free_port(), out), nprocs=world, start_method="spawn")
        r = np.load(out)
        assert r["slabbed"].shape == r["ref"].shape
        assert np.array_equal(r["slabbed"], r["ref"])


def test_decomposition_rows_and_neighbours():
    import obgc
    g = obgc.RectilinearGrid((8, 12, 4), (800.0, 1200.0, 40.0))
    d = obgc.SlabDecomposition(g, 0, 3)
    assert (d.south, d.north, d.Ny_own) == (2, 1, 4)
    assert list(d.global_rows()) == [9, 10, 11, 0, 1, 2, 3, 4, 5, 6]
    assert d.slab_grid.Ny == 10 and abs(d.slab_grid.Ly / d.slab_grid.Ny - g.Ly / g.Ny) < 1e-12
    with pytest.raises(ValueError):
        obgc.SlabDecomposition(g, 0, 5)                 # 12 rows do not split in 5
    with pytest.raises(ValueError):
        obgc.SlabDecomposition(g, 0, 6)                 # 2 own rows < the 3-row halo
    with pytest.raises(ValueError):
        obgc.SlabDecomposition(obgc.RectilinearGrid((8, 12, 4), (1.0, 1.0, 1.0), ("Periodic", "Bounded", "Bounded")), 0, 2)


def test_single_rank_exchange_wraps_onto_itself():
    import obgc
    g = obgc.RectilinearGrid((4, 6, 2), (4.0, 6.0, 2.0))
    d = obgc.SlabDecomposition(g, 0, 1)
    field = np.arange(2 * 6 * 4, dtype=np.float64).reshape(1, 2, 6, 4)
    st = np.stack([d.scatter(field[0])])
    ss, sn = pack_rows(st, d)
    rs, rn = torch.empty(d.buffer_shape(1), dtype=torch.float64), torch.empty(d.buffer_shape(1), dtype=torch.float64)
    d.exchange(torch.from_numpy(ss), torch.from_numpy(sn), rs, rn)
    unpack_rows(st, d, rs.numpy(), rn.numpy())
    assert np.array_equal(st, np.stack([d.scatter(field[0])]))


PISCES_SHAPE, PISCES_STEPS, PISCES_DT = (16, 12, 10), 2, 600.0


def pisces_case(grid_shape=PISCES_SHAPE):
    import obgc
    g = obgc.RectilinearGrid(grid_shape, (16000.0, 12000.0, 500.0), ("Periodic", "Periodic", "Bounded"))
    bgc = obgc.PISCES(g)
    light = obgc.MultiBandPhotosyntheticallyActiveRadiation(grid=g, surface_PAR=100.0)
    u, v, _ = obgc.random_streamfunction_velocity(g, rms=0.1, seed=4, device="cpu", dtype=torch.float64)
    init = obgc.pisces_initial_conditions(g, seed=6)
    from obgc import _abi as A
    state0 = np.ascontiguousarray(np.stack([np.broadcast_to(init[n], g.shape) for n in A.PISCES_ASCII]).astype(np.float64))
    return g, bgc, light, u.numpy(), v.numpy(), state0


def pisces_oracle_model(bgc, grid, light):
    import oracle as O
    from obgc import _abi as A
    return O.pisces3d(bgc.params, grid.c_grid(), light, -60.0, surface_kind=A.SURFACE_CONSTANT, surface_value=100.0)


def pisces_rank_main(rank, world, port, out_path):
    import oracle as O
    import obgc
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        g, bgc, light, u, v, state0 = pisces_case()
        d = obgc.SlabDecomposition(g, rank, world)
        m = pisces_oracle_model(bgc, d.slab_grid, light)
        st = np.ascontiguousarray(np.stack([d.scatter(state0[q]) for q in range(state0.shape[0])]))
        us = np.ascontiguousarray(d.scatter(u).ravel())
        vs = np.ascontiguousarray(d.scatter(v).ravel())
        G, Gm = np.zeros_like(st), np.zeros_like(st)
        rs = torch.empty(d.buffer_shape(st.shape[0]), dtype=torch.float64)
        rn = torch.empty_like(rs)
        for n in range(PISCES_STEPS):
            for stage in range(3):
                ss, sn = pack_rows(st, d)
                d.exchange(torch.from_numpy(ss), torch.from_numpy(sn), rs, rn)
                unpack_rows(st, d, rs.numpy(), rn.numpy())
                O.pisces_stage3d(m, st, G, Gm, u=us, v=vs, t=n * PISCES_DT, dt=PISCES_DT, stage=stage,
                                 start=(n == 0 and stage == 0), threads=1)
                G, Gm = Gm, G
        own = torch.from_numpy(np.ascontiguousarray(st[:, :, d.own(), :]))
        parts = [torch.empty_like(own) for _ in range(world)] if rank == 0 else None
        dist.gather(own, parts, dst=0)
        if rank == 0:
            slabbed = torch.cat(parts, dim=2).numpy()
            ref = state0.copy()
            O.pisces_step3d(pisces_oracle_model(bgc, g, light), ref, u=u.ravel().copy(), v=v.ravel().copy(), t=0.0,
                            dt=PISCES_DT, nsteps=PISCES_STEPS, threads=1)
            np.savez(out_path, slabbed=slabbed, ref=ref)
    finally:
        dist.destroy_process_group()


def test_pisces_slabbed_oracle_with_exchanged_halos_equals_single_domain():
    # configuration 4's model: two gloo ranks, each stepping its slab with the oracle's PISCES stage
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "result.npz")
        mp.start_processes(pisces_rank_main, args=(2, free_port(), out), nprocs=2, start_method="spawn")
        r = np.load(out)
        assert r["slabbed"].shape == r["ref"].shape
        assert np.array_equal(r["slabbed"], r["ref"])


def test_shard_runs_balances_and_covers_every_run():
    import obgc
    costs = [5, 1, 9, 3, 3, 7, 2, 8]
    shards = obgc.shard_runs(costs, 3)
    assert sorted(q for s in shards for q in s) == list(range(len(costs)))
    loads = [sum(costs[q] for q in s) for s in shards]
    assert max(loads) - min(loads) <= max(costs)
    assert obgc.shard_runs(costs, 3) == shards             # the same on every rank
    assert obgc.shard_runs(costs, 1) == [list(range(len(costs)))]


def columns_rank_main(rank, world, port, out_path):
    import obgc
    from test_oracle_columns import run as run_columns
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        bgc = obgc.NPZD(None)
        cols = obgc.npzd_column_ensemble(9, seed=5, levels=(16, 64), nsteps=30)
        names = obgc.required_biogeochemical_tracers(bgc)
        shards = obgc.shard_runs([c["init"].shape[1] * c["nsteps"] for c in cols], world)
        mine = [cols[q] for q in shards[rank]]
        local = run_columns(bgc, mine, names) if mine else []
        got = obgc.gather_runs(local, shards)
        if rank == 0:
            ref = run_columns(bgc, cols, names)
            np.savez(out_path, ok=np.array([np.array_equal(a, b) for a, b in zip(got, ref)]),
                     n=np.array([len(s) for s in shards]))
    finally:
        dist.destroy_process_group()


def test_column_runs_sharded_over_ranks_equal_one_rank():
    # columns are independent runs: two gloo ranks each run their shard (the oracle's column runner
    # standing in for the column engine), rank 0 gathers them in the global order
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "result.npz")
        mp.start_processes(columns_rank_main, args=(2, free_port(), out), nprocs=2, start_method="spawn")
        r = np.load(out)
        assert r["ok"].all() and len(r["ok"]) == 9 and (r["n"] > 0).all()
