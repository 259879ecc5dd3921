"""Computational grid: spacing, time step and sizes (mirrors ``fullwave/grid.py:44-147``)."""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Grid:
    """Uniform grid with ``dx = c0 / f0 / ppw`` and ``dt = cfl * dx / c0``.

    Same fields, properties and input checks as the reference ``Grid`` (grid.py:44-70,
    :115-147), so the engine sees the same ``nX, nY, nZ, nT, dX, dY, dZ, dT``.
    """

    domain_size: tuple
    f0: float
    duration: float
    c0: float = 1540
    ppw: int = 12
    cfl: float = 0.2

    def __post_init__(self) -> None:
        assert len(self.domain_size) in (2, 3), "Domain size must be 2D or 3D"
        assert self.f0 > 0, "Center frequency must be greater than 0"
        assert self.f0 < 30e6, "Center frequency must be less than 30 MHz"
        assert self.duration > 0, "Duration must be greater than 0"
        assert self.c0 > 0, "Speed of sound must be greater than 0"
        assert self.ppw > 5, "Points per wavelength must be greater than 5"
        assert self.cfl > 0.01, "CFL number must be greater than 0.01"
        assert self.cfl < 0.5, "CFL number must be less than 0.5"
        self.is_3d = len(self.domain_size) == 3

    @property
    def omega(self) -> float:
        return 2 * np.pi * self.f0

    @property
    def wavelength(self) -> float:
        return self.c0 / self.f0

    @property
    def dx(self) -> float:
        return self.wavelength / self.ppw

    @property
    def dy(self) -> float:
        return self.wavelength / self.ppw

    @property
    def dz(self) -> float:
        return self.wavelength / self.ppw if self.is_3d else 0

    @property
    def dt(self) -> float:
        return self.cfl * self.dx / self.c0

    @property
    def nx(self) -> int:
        return int(np.round(self.domain_size[0] / self.dx).item())

    @property
    def ny(self) -> int:
        return int(np.round(self.domain_size[1] / self.dy).item())

    @property
    def nz(self) -> int:
        return int(np.round(self.domain_size[2] / self.dz).item()) if self.is_3d else 0

    @property
    def nt(self) -> int:
        return round(self.duration / self.dt)

    @property
    def shape(self) -> tuple:
        return (self.nx, self.ny, self.nz) if self.is_3d else (self.nx, self.ny)

    @classmethod
    def from_cells(cls, shape, *, f0: float, nt: int, c0: float = 1540, ppw: int = 12,
                   cfl: float = 0.2) -> "Grid":
        """Grid whose ``shape`` and ``nt`` are the given cell and step counts."""
        dx = c0 / f0 / ppw
        dt = cfl * dx / c0
        return cls(domain_size=tuple(n * dx for n in shape), f0=f0, duration=nt * dt, c0=c0,
                   ppw=ppw, cfl=cfl)
