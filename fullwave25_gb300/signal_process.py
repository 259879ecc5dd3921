"""Output formats on the far side of the engine: whole-domain sensor traces reshaped into
wavefield movies, and the signed power compression used to display them.

Restates ``fullwave/utils/signal_process.py`` (``signed_power_compression`` :13-33,
``reshape_whole_sensor_to_nx_ny_nt`` :35-58, ``reshape_whole_sensor_to_nt_nx_ny`` :61-115,
``reshape_whole_sensor_to_nt_nx_ny_nz`` :145-205). The input is what
``Solver.run(record_whole_domain=True)`` returns: ``[n_sensors, n_out]`` with the sensors in the
C order of the (extended) grid, x slowest.
"""

from __future__ import annotations

import numpy as np


def signed_power_compression(x, power: float = 1 / 3):
    """``sign(x) |x|^power`` (keeps the sign, compresses the dynamic range)."""
    x = np.asarray(x)
    return np.sign(x) * np.abs(x) ** power


def _dims(grid, names, given, use_grid):
    if grid is not None and any(v is not None for v in given[:2]):
        raise ValueError("Either grid or both nx and ny must be provided, not both.")
    if use_grid:
        return tuple(int(getattr(grid, n)) for n in names)
    if any(v is None for v in given):
        raise ValueError("Either grid or both nx and ny must be provided.")
    return tuple(int(v) for v in given)


def reshape_whole_sensor_to_nx_ny_nt(sensor_output, grid):
    """``[n_sensors, nt]`` -> ``[nx, ny, nt]``, read with the reference's (ny, nx) split of the
    sensor axis followed by an axis swap (signal_process.py:35-58)."""
    a = np.asarray(sensor_output)
    return a.reshape((int(grid.ny), int(grid.nx), a.shape[-1])).transpose(1, 0, 2)


def reshape_whole_sensor_to_nt_nx_ny(sensor_output, grid=None, nx=None, ny=None, *,
                                     use_grid: bool = True):
    """``[n_sensors, nt]`` -> ``[nt, nx, ny]`` (sensor k = i * ny + j)."""
    a = np.asarray(sensor_output)
    nx, ny = _dims(grid, ("nx", "ny"), (nx, ny), use_grid)
    return a.reshape((nx, ny, a.shape[-1])).transpose(2, 0, 1)


def reshape_whole_sensor_to_nt_nx_ny_nz(sensor_output, grid=None, nx=None, ny=None, nz=None, *,
                                        use_grid: bool = True):
    """``[n_sensors, nt]`` -> ``[nt, nx, ny, nz]`` (sensor k = (i * ny + j) * nz + l)."""
    a = np.asarray(sensor_output)
    nx, ny, nz = _dims(grid, ("nx", "ny", "nz"), (nx, ny, nz), use_grid)
    return a.reshape((nx, ny, nz, a.shape[-1])).transpose(3, 0, 1, 2)
