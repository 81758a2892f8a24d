"""A 3-D model split across GPUs in y slabs (the reference runs one NonhydrostaticModel per MPI rank
on Oceananigans' Distributed architecture, whose fill_halo_regions! exchanges halo rows before
each tendency computation).

Rank r of W owns rows [r Ny/W, (r + 1) Ny/W) of a Periodic-y grid.  Its slab is a grid of
Ny/W + 2H rows (H = 3, the WENO5 stencil's reach) with the same dx, dy and dz, also Periodic in y:
the fused kernels then read every stencil of an own row from the slab itself, and the halo rows'
own updates (which wrap inside the slab) are overwritten by the next exchange.  Light, pH and the
sediment are column-local, so the only exchange is H rows of every tracer before each RK3 stage:
each rank packs its first and last H own rows (obgc_halo_pack), sends them to its southern and
northern neighbours and unpacks what they sent into its halo rows (obgc_halo_unpack).  The sends
go into each rank's own receive buffers (torch.distributed point-to-point: NCCL on GPUs, gloo on
CPU ranks); no collective is on the data path.
"""
import ctypes as C

import numpy as np

from . import _abi as A
from .grid import RectilinearGrid

HALO = 3
TAG_SOUTHWARD, TAG_NORTHWARD = 17, 18


class SlabDecomposition:
    """Rows, neighbours and the slab grid of one rank."""

    def __init__(self, grid, rank, world, halo=HALO):
        if grid.topology[1] != "Periodic":
            raise ValueError("the y slab split needs a Periodic y direction")
        if grid.Ny % world != 0:
            raise ValueError(f"Ny = {grid.Ny} does not split into {world} equal slabs")
        self.grid, self.rank, self.world, self.halo = grid, rank, world, halo
        self.Ny_own = grid.Ny // world
        if self.Ny_own < halo:
            raise ValueError(f"a slab needs at least {halo} own rows")
        self.j0 = rank * self.Ny_own
        self.south = (rank - 1) % world
        self.north = (rank + 1) % world
        ny = self.Ny_own + 2 * halo
        self.slab_grid = RectilinearGrid((grid.Nx, ny, grid.Nz), (grid.Lx, grid.Ly * ny / grid.Ny, grid.Lz),
                                         grid.topology, dtype=grid.dtype)

    def global_rows(self):
        """Global row of each slab row (halos wrap around the periodic domain)."""
        return (self.j0 - self.halo + np.arange(self.Ny_own + 2 * self.halo)) % self.grid.Ny

    def own(self):
        """Slice of the slab's own rows along y."""
        return slice(self.halo, self.halo + self.Ny_own)

    def scatter(self, field):
        """A global (Nz, Ny, Nx) field's rows of this slab, halos included (numpy or torch)."""
        rows = self.global_rows()
        if hasattr(field, "index_select"):
            import torch
            return field.index_select(1, torch.as_tensor(rows, device=field.device)).contiguous()
        return np.ascontiguousarray(np.asarray(field)[:, rows, :])

    def buffer_shape(self, n_fields):
        return (n_fields, self.grid.Nz, self.halo, self.grid.Nx)

    def exchange(self, send_south, send_north, recv_south, recv_north, group=None):
        """Send this rank's first own rows south and last own rows north; receive the southern
        neighbour's last rows into recv_south and the northern neighbour's first rows into
        recv_north.  One rank: the periodic wrap onto itself."""
        if self.world == 1:
            recv_south.copy_(send_north)
            recv_north.copy_(send_south)
            return
        import torch.distributed as dist
        ops = [dist.P2POp(dist.isend, send_south, self.south, group, TAG_SOUTHWARD),
               dist.P2POp(dist.isend, send_north, self.north, group, TAG_NORTHWARD),
               dist.P2POp(dist.irecv, recv_north, self.north, group, TAG_SOUTHWARD),
               dist.P2POp(dist.irecv, recv_south, self.south, group, TAG_NORTHWARD)]
        for r in dist.batch_isend_irecv(ops):
            r.wait()


class SlabModel:
    """One rank's slab of a NonhydrostaticModel split in y: the slab model (the library's fused RK3
    stages on the slab grid), a second set of state arrays for the stage ping-pong, and the halo
    buffers.  `exchange` moves the packed buffers between ranks (default: the decomposition's
    torch.distributed exchange)."""

    def __init__(self, decomposition, biogeochemistry, velocities, initial, tracers=("T", "S"), precision="f32",
                 exchange=None, **model_kw):
        import torch
        from .model3d import NonhydrostaticModel, set_
        self.decomposition = d = decomposition
        u, v, w = velocities
        self.model = NonhydrostaticModel(d.slab_grid, biogeochemistry=biogeochemistry, tracers=tracers,
                                         velocities=(d.scatter(u), d.scatter(v), None if w is None else d.scatter(w)),
                                         precision=precision, **model_kw)
        set_(self.model, **{k: (d.scatter(np.broadcast_to(np.asarray(x, dtype=np.float64), d.grid.shape))
                                if not isinstance(x, (int, float)) else x) for k, x in initial.items()})
        m = self.model
        self.names = list(m.tracer_names)
        self.fields = [m.tracers[n] for n in self.names]
        self.other = [torch.empty_like(f) for f in self.fields]
        shape = d.buffer_shape(len(self.names))
        dt = m.state_dtype
        self.send = [torch.empty(shape, dtype=dt, device=m.device) for _ in range(2)]
        self.recv = [torch.empty(shape, dtype=dt, device=m.device) for _ in range(2)]
        self.exchange = exchange or (lambda ss, sn, rs, rn: d.exchange(ss, sn, rs, rn))
        self._lib = A.load()
        self._cgrid = d.slab_grid.c_grid()
        self._dtype = A.F32 if dt == torch.float32 else A.F64
        self.cur = self.nxt = None

    def _ptrs(self, fields):
        return (C.c_void_p * len(fields))(*[f.data_ptr() for f in fields])

    def pack(self, fields):
        A.check(self._lib.obgc_halo_pack(C.byref(self._cgrid), self._dtype, len(fields), self._ptrs(fields),
                                         self.decomposition.halo, self.send[0].data_ptr(), self.send[1].data_ptr(),
                                         self.model._stream()), "obgc_halo_pack")

    def unpack(self, fields):
        A.check(self._lib.obgc_halo_unpack(C.byref(self._cgrid), self._dtype, len(fields), self._ptrs(fields),
                                           self.decomposition.halo, self.recv[0].data_ptr(), self.recv[1].data_ptr(),
                                           self.model._stream()), "obgc_halo_unpack")

    def substep(self, stage, dt, cur, nxt):
        m = self.model
        A.check(self._lib.obgc_substep(m._ctx, m.clock.time, float(dt), int(stage), self._ptrs(cur), self._ptrs(nxt),
                                       m._stream()), "obgc_substep")

    # One RK3 stage is pack_halos(), exchange_halos() (between all ranks), then run_stage(); the
    # state ping-pongs between the model's arrays and `other` (self.cur holds it).
    def pack_halos(self):
        if self.cur is None:
            self.cur, self.nxt = self.fields, self.other
        self.pack(self.cur)

    def exchange_halos(self):
        self.exchange(self.send[0], self.send[1], self.recv[0], self.recv[1])

    def run_stage(self, stage, dt):
        self.unpack(self.cur)
        self.substep(stage, dt, self.cur, self.nxt)
        self.cur, self.nxt = self.nxt, self.cur
        if stage == 2:
            self.model.clock.time += dt
            self.model.clock.iteration += 1

    def sync_fields(self):
        """Leave the state in the model's own tracer arrays."""
        if self.cur is not None and self.cur is not self.fields:
            for a, b in zip(self.fields, self.cur):
                a.copy_(b)
        self.cur = None

    def time_step(self, dt, nsteps=1):
        """nsteps RK3 steps: before every stage the halos are exchanged, then the stage runs on the
        slab.  The result lands in the model's own tracer arrays."""
        for _ in range(nsteps):
            for stage in range(3):
                self.pack_halos()
                self.exchange_halos()
                self.run_stage(stage, dt)
        self.sync_fields()

    def own_state(self):
        """(n_tracers, Nz, Ny_own, Nx) of the slab's own rows."""
        import torch
        src = self.cur if self.cur is not None else self.fields
        return torch.stack([f[:, self.decomposition.own(), :] for f in src])


class PiscesSlabModel:
    """One rank's slab of a PISCES 3-D model split in y (configuration 4): a PiscesModel on the slab
    grid, a second set of state arrays for the stage ping-pong and the halo buffers; the stage loop
    is SlabModel's.  Light, the euphotic depth, the mixed-layer means and the calcite saturation are
    column-local, so the halo rows of the 26 tracers are the only exchange."""

    def __init__(self, decomposition, velocities, initial, precision="f32", exchange=None, **model_kw):
        import torch
        from .pisces import PiscesModel
        self.decomposition = d = decomposition
        u, v = velocities[:2]
        self.model = PiscesModel(d.slab_grid, velocities=(d.scatter(u), d.scatter(v)), precision=precision, **model_kw)
        self.model.set_(**{k: d.scatter(np.broadcast_to(np.asarray(x, dtype=np.float64), d.grid.shape))
                           for k, x in initial.items()})
        m = self.model
        self.names = list(A.PISCES_TRACERS)
        self.fields = [m.tracers[n] for n in self.names]
        self.other = [torch.empty_like(f) for f in self.fields]
        shape = d.buffer_shape(len(self.names))
        dev = self.fields[0].device
        self.send = [torch.empty(shape, dtype=m.dtype, device=dev) for _ in range(2)]
        self.recv = [torch.empty(shape, dtype=m.dtype, device=dev) for _ in range(2)]
        self.exchange = exchange or (lambda ss, sn, rs, rn: d.exchange(ss, sn, rs, rn))
        self._lib = A.load()
        self._cgrid = d.slab_grid.c_grid()
        self._dtype = A.F32 if m.dtype == torch.float32 else A.F64
        self.cur = self.nxt = None
        self._last_stage = False

    def _ptrs(self, fields):
        return (C.c_void_p * len(fields))(*[f.data_ptr() for f in fields])

    @staticmethod
    def _stream():
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream) if torch.cuda.is_available() else None

    def pack(self, fields):
        A.check(self._lib.obgc_halo_pack(C.byref(self._cgrid), self._dtype, len(fields), self._ptrs(fields),
                                         self.decomposition.halo, self.send[0].data_ptr(), self.send[1].data_ptr(),
                                         self._stream()), "obgc_halo_pack")

    def unpack(self, fields):
        A.check(self._lib.obgc_halo_unpack(C.byref(self._cgrid), self._dtype, len(fields), self._ptrs(fields),
                                           self.decomposition.halo, self.recv[0].data_ptr(), self.recv[1].data_ptr(),
                                           self._stream()), "obgc_halo_unpack")

    def pack_halos(self):
        if self.cur is None:
            self.cur, self.nxt = self.fields, self.other
        self.pack(self.cur)

    def exchange_halos(self):
        self.exchange(self.send[0], self.send[1], self.recv[0], self.recv[1])

    def run_stage(self, stage, dt, finish=False):
        """finish: this is the call's last stage (obgc_pisces_model_step applies the negative-tracer
        modifier after it)."""
        m = self.model
        self.unpack(self.cur)
        A.check(self._lib.obgc_pisces_model_substep(m._h, float(m.time), float(dt), int(stage), self._ptrs(self.cur),
                                                    self._ptrs(self.nxt), int(bool(finish)), self._stream()),
                "obgc_pisces_model_substep")
        self.cur, self.nxt = self.nxt, self.cur
        if stage == 2:
            m.time += dt

    def sync_fields(self):
        if self.cur is not None and self.cur is not self.fields:
            for a, b in zip(self.fields, self.cur):
                a.copy_(b)
        self.cur = None

    def time_step(self, dt, nsteps=1):
        for s in range(nsteps):
            for stage in range(3):
                self.pack_halos()
                self.exchange_halos()
                self.run_stage(stage, dt, finish=(s == nsteps - 1 and stage == 2))
        self.sync_fields()

    def own_state(self):
        """(26, Nz, Ny_own, Nx) of the slab's own rows."""
        import torch
        src = self.cur if self.cur is not None else self.fields
        return torch.stack([f[:, self.decomposition.own(), :] for f in src])


def shard_runs(costs, world):
    """Independent runs (columns, service requests, box models) shared out over `world` ranks: the
    largest cost first, each to the least-loaded rank so far (ties to the lower rank), so that the
    ranks' work is balanced and the assignment is the same on every rank.  costs: one number per run
    (e.g. levels x steps).  Returns, per rank, the sorted indices of its runs."""
    order = sorted(range(len(costs)), key=lambda q: (-float(costs[q]), q))
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for q in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(q)
        load[r] += float(costs[q])
    return [sorted(x) for x in out]


def gather_runs(local_results, shards, group=None):
    """Rank 0 receives every rank's results (a list in the order of that rank's shard) and returns
    them in the runs' global order; other ranks return None.  One rank: the results as they are."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return list(local_results)
    parts = [None] * dist.get_world_size(group) if dist.get_rank(group) == 0 else None
    dist.gather_object(list(local_results), parts, dst=0, group=group)
    if parts is None:
        return None
    out = [None] * sum(len(s) for s in shards)
    for shard, res in zip(shards, parts):
        for q, x in zip(shard, res):
            out[q] = x
    return out
