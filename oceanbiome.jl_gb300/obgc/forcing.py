"""Tracer forcing of the fused 3-D step: a prescribed source-rate field, optionally switched on over
a window of time.

Oceananigans' `forcing = (; X = Forcing(func; parameters))` evaluates a function of (x, y, z, t) in
the tendency kernel.  Here the spatial part is a field sampled once on the grid's cell centres and
the time dependence is a window [start_time, end_time) tested against each RK3 stage's clock; the
alkalinity release of examples/oae_experiment.jl:55-79 (a rate inside a disc near the surface
between two times) is exactly such a forcing.
"""
import math

import numpy as np


class Forcing:
    """Forcing(rate; start_time=-inf, end_time=inf): `rate` is a number, a numpy array or tensor of the
    grid's shape (Nz, Ny, Nx), or a function f(x, y, z) sampled at the cell centres; tracer units per
    second."""

    def __init__(self, rate, start_time=-math.inf, end_time=math.inf):
        if not end_time >= start_time:
            raise ValueError("Forcing: end_time before start_time")
        self.rate, self.start_time, self.end_time = rate, float(start_time), float(end_time)

    def field(self, grid, dtype, device):
        """The rate as a device tensor of the grid's shape."""
        import torch
        r = self.rate
        if callable(r):
            z, y, x = grid.nodes()
            r = np.vectorize(r)(x[None, None, :], y[None, :, None], z[:, None, None])
        if isinstance(r, (int, float)):
            return torch.full(grid.shape, float(r), dtype=dtype, device=device)
        t = torch.as_tensor(np.asarray(r) if not isinstance(r, torch.Tensor) else r)
        return torch.broadcast_to(t, grid.shape).to(device=device, dtype=dtype).contiguous()
