"""Problem definitions and model generation (host side, no GPU needed).

A `Problem` fixes the grid (interior n, `bord`, `absorb` shells as in
original/main.c:95-97), spacing, time step, step count, source (position and
cut frequency) and medium; `model()` builds the six model arrays with the
library's host generators and applies the random-velocity boundary
(original/boundary.c:7-98) after srand(seed).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

from . import _lib
from ._lib import fptr


@dataclass(frozen=True)
class Problem:
    name: str
    nx: int
    ny: int
    nz: int
    absorb: int
    bord: int = 4
    dx: float = 12.5
    dy: float = 12.5
    dz: float = 12.5
    dt: float = 0.001
    steps: int = 200
    fcut: float = 40.0            # Ricker cut frequency; peak = fcut / 3
    kind: str = "homogeneous"     # or "layered"
    seed: int = 1                 # srand() seed of the boundary draws (and layered draws)
    medium: tuple = (3000.0, 1500.0, 0.24, 0.10, math.pi / 6, math.pi / 4)  # vpz vsv eps delta phi theta
    layers: int = 8
    vrange: tuple = (1500.0, 4000.0)
    vs_ratio: float = 0.5
    source: tuple | None = None   # (ix, iy, iz) in full-grid indices; None = centre

    @property
    def sx(self) -> int:
        return self.nx + 2 * self.bord + 2 * self.absorb

    @property
    def sy(self) -> int:
        return self.ny + 2 * self.bord + 2 * self.absorb

    @property
    def sz(self) -> int:
        return self.nz + 2 * self.bord + 2 * self.absorb

    @property
    def n(self) -> int:
        return self.sx * self.sy * self.sz

    @property
    def updated_cells(self) -> int:
        """Cells one step updates: the reference's samplesPropagate (original/model.c:44)."""
        b = self.bord
        return (self.sx - 2 * b) * (self.sy - 2 * b) * (self.sz - 2 * b)

    @property
    def src_xyz(self) -> tuple:
        return self.source if self.source is not None else (self.sx // 2, self.sy // 2, self.sz // 2)

    @property
    def i_source(self) -> int:
        ix, iy, iz = self.src_xyz
        return (iz * self.sy + iy) * self.sx + ix

    def with_(self, **kw) -> "Problem":
        return replace(self, **kw)

    def raw_model(self) -> np.ndarray:
        """(6, n) float32 before the boundary: vpz vsv epsilon delta phi theta."""
        lib = _lib.load()
        m = np.empty((6, self.n), np.float32)
        if self.kind == "homogeneous":
            lib.FLETCHER_ModelHomogeneous(self.n, *[float(v) for v in self.medium], fptr(m))
        elif self.kind == "layered":
            lib.FLETCHER_ModelLayered(self.sx, self.sy, self.sz, self.bord, self.absorb, self.layers,
                                      self.seed, float(self.vrange[0]), float(self.vrange[1]),
                                      float(self.vs_ratio), fptr(m), None)
        else:
            raise ValueError(self.kind)
        return m

    def model(self) -> np.ndarray:
        """(6, n) float32 with the random-velocity boundary applied."""
        lib = _lib.load()
        m = self.raw_model()
        lib.FLETCHER_RandomVelocityBoundary(self.sx, self.sy, self.sz, self.nx, self.ny, self.nz, self.bord,
                                            self.absorb, fptr(m[0]), fptr(m[1]), self.seed)
        return m

    def sources(self, steps: int | None = None) -> np.ndarray:
        """Source values for steps it = 1..steps (time (it-1)*dt), original/model.c:74."""
        lib = _lib.load()
        st = self.steps if steps is None else steps
        return np.array([lib.FLETCHER_Source(self.dt, it, self.fcut) for it in range(st)], np.float32)


# The configurations the project is measured on.
C0 = Problem("C0-homogeneous-56", 56, 56, 56, absorb=16, dt=0.001, steps=200, fcut=60.0,
             medium=(3000.0, 1500.0, 0.24, 0.10, math.radians(30.0), math.radians(45.0)))


def _layered(name, n, steps, absorb=32, dt=0.0006, seed=1):
    bord = 4
    s = n + 2 * bord + 2 * absorb
    return Problem(name, n, n, n, absorb=absorb, bord=bord, dt=dt, steps=steps, fcut=45.0, kind="layered",
                   seed=seed, source=(s // 2, s // 2, bord + absorb + 8))


C1 = _layered("C1-layered-504", 504, 1000)
C2 = _layered("C2-layered-128", 128, 2000)
