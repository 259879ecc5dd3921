"""Pressure source and sensor descriptions (mirror ``fullwave/source.py`` and ``fullwave/sensor.py``)."""

from __future__ import annotations

import numpy as np

from .coords import coords_to_map, map_to_coords


class Source:
    """Time-varying pressure at the cells of ``mask``.

    ``p0`` is ``[n_sources, nt]``; its rows follow :func:`map_to_coords` order (source.py:25-77).
    The engine drives ``p`` at ``incoords[k]`` with ``p0[k, n]`` for every step ``n < nt``.
    """

    def __init__(self, p0: np.ndarray, mask: np.ndarray) -> None:
        self.p0 = np.atleast_2d(p0)
        mask = np.atleast_2d(mask)
        self.grid_shape = mask.shape
        self.is_3d = len(self.grid_shape) == 3
        self.incoords = map_to_coords(mask)
        if self.p0.shape[0] != self.incoords.shape[0]:
            raise ValueError("Input signal has the wrong number of elements")

    @property
    def icmat(self) -> np.ndarray:
        return self.p0

    @property
    def mask(self) -> np.ndarray:
        return coords_to_map(self.incoords, self.grid_shape)

    @property
    def n_sources(self) -> int:
        return int(self.incoords.shape[0])

    ncoords = n_sources

    def validate(self, grid_shape) -> None:
        assert tuple(self.grid_shape) == tuple(grid_shape), f"{self.grid_shape} != {tuple(grid_shape)}"
        assert self.n_sources > 0, "No active source found."


class Sensor:
    """Cells whose pressure is recorded every ``sampling_modulus_time`` steps (sensor.py:24-94)."""

    def __init__(self, mask: np.ndarray, sampling_modulus_time: int = 1) -> None:
        mask = np.atleast_2d(mask)
        self.grid_shape = mask.shape
        self.sampling_modulus_time = int(sampling_modulus_time)
        self.is_3d = len(self.grid_shape) == 3
        self.outcoords = map_to_coords(mask)

    @property
    def mask(self) -> np.ndarray:
        return coords_to_map(self.outcoords, self.grid_shape)

    @property
    def n_sensors(self) -> int:
        return int(self.outcoords.shape[0])

    ncoordsout = n_sensors

    def validate(self, grid_shape) -> None:
        assert tuple(self.grid_shape) == tuple(grid_shape), f"{self.grid_shape} != {tuple(grid_shape)}"
        assert self.n_sensors > 0, "No active sensor found."
