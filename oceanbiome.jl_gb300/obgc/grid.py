"""RectilinearGrid mirror: sizes, extents, topology and the field layout handed to the C ABI."""
import numpy as np

from . import _abi as A

_TOPO = {"Periodic": A.PERIODIC, "Bounded": A.BOUNDED, "Flat": A.FLAT}


class RectilinearGrid:
    """Uniform rectilinear grid, k = 0 at the bottom.  size/extent follow Oceananigans:
    (Nx, Ny, Nz) / (Lx, Ly, Lz); a Flat direction takes size 1 and any extent.  Fields are
    dense i-fastest tensors of shape (Nz, Ny, Nx)."""

    def __init__(self, size, extent, topology=("Periodic", "Periodic", "Bounded"), dtype="f64"):
        if len(size) == 2:   # (Nx, Nz) for (Bounded/Periodic, Flat, Bounded)
            size = (size[0], 1, size[1])
            extent = (extent[0], 1.0, extent[1])
        self.Nx, self.Ny, self.Nz = (int(x) for x in size)
        self.Lx, self.Ly, self.Lz = (float(x) for x in extent)
        self.topology = tuple(topology)
        if self.topology[2] != "Bounded":
            raise ValueError("the vertical direction must be Bounded")
        self.dtype = dtype

    @property
    def shape(self):
        return (self.Nz, self.Ny, self.Nx)

    @property
    def N(self):
        return self.Nx * self.Ny * self.Nz

    @property
    def dz(self):
        return self.Lz / self.Nz

    def znodes(self, loc="center"):
        zf = -self.Lz + self.dz * np.arange(self.Nz + 1)
        return zf if loc == "face" else zf[:-1] + self.dz / 2

    def nodes(self):
        """Cell-centre coordinates (z, y, x): x in (0, Lx), y in (0, Ly), z in (-Lz, 0), as
        Oceananigans places a grid of the given extent; a Flat direction gives 0."""
        x = (np.arange(self.Nx) + 0.5) * (self.Lx / self.Nx) if self.topology[0] != "Flat" else np.zeros(1)
        y = (np.arange(self.Ny) + 0.5) * (self.Ly / self.Ny) if self.topology[1] != "Flat" else np.zeros(1)
        return self.znodes(), y, x

    def c_grid(self, stride_j=None, stride_k=None):
        g = A.Grid()
        g.Nx, g.Ny, g.Nz = self.Nx, self.Ny, self.Nz
        g.topology_x, g.topology_y = _TOPO[self.topology[0]], _TOPO[self.topology[1]]
        g.Lx, g.Ly, g.Lz = self.Lx, self.Ly, self.Lz
        g.stride_j = self.Nx if stride_j is None else stride_j
        g.stride_k = self.Nx * self.Ny if stride_k is None else stride_k
        return g


def BoxModelGrid():
    """src/OceanBioME.jl:171: a single point."""
    return RectilinearGrid((1, 1, 1), (1.0, 1.0, 1.0), ("Flat", "Flat", "Bounded"))
