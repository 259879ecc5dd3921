"""Mask <-> coordinate conversion with the reference's row-major ordering.

``map_to_coords`` follows ``fullwave/utils/coordinates.py:28-53``: the coordinates of the
non-zero cells in C (row-major) order, one row per cell, columns ``(x, y[, z])``. This order is
the order of the rows of ``icmat`` and of the columns of the returned sensor traces.
"""

from __future__ import annotations

import numpy as np


def map_to_coords(mask: np.ndarray) -> np.ndarray:
    """Coordinates ``[n, ndim]`` (int64) of the non-zero cells of ``mask`` in row-major order."""
    return np.array([*np.where(np.asarray(mask) != 0)]).T.astype(np.int64).reshape(-1, np.ndim(mask))


def coords_to_map(coords: np.ndarray, grid_shape) -> np.ndarray:
    """Inverse of :func:`map_to_coords` (coordinates.py:56-85)."""
    out = np.zeros(tuple(grid_shape), dtype=int)
    c = np.asarray(coords).astype(int)
    if c.size:
        out[tuple(c[:, k] for k in range(c.shape[1]))] = 1
    return out
