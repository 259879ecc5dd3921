"""Exponential-attenuation medium and its PML (the reference's third engine family).

Mirrors ``fullwave/medium.py:560-750`` (``MediumExponentialAttenuation``), the conversion
``Medium._db_mhz_cm_to_a_exp`` (medium.py:1068-1090) and ``PMLBuilderExponentialAttenuation``
(fullwave/solver/pml_builder.py:1652-1935):

* ``a_exp = exp(-dt * texp)`` with ``texp = alpha0 / 2 * f0[MHz] * c0 / (1e-2 * 8.686...)``:
  the fraction of amplitude kept per time step by each of the two field updates;
* the grid is padded by ``n_pml + 8`` cells (edge values for every map, the air map included,
  as pml_builder.py:1768-1778 does), and inside the padding ``a_exp`` is scaled by ``1 - r``,
  ``r`` the normalised distance into the padding (pml_builder.py:1800-1935).
"""

from __future__ import annotations

import numpy as np

from .coefficients import N_TAPS
from .grid import Grid
from .pml import extend_map
from .source import Sensor, Source


def db_mhz_cm_to_a_exp(alpha_coeff, grid: Grid) -> np.ndarray:
    np_factor = -10 * np.log10(np.exp(-1))
    f0 = grid.omega / (2.0 * np.pi * 1e6) if hasattr(grid, "omega") else grid.f0 / 1e6
    texp = np.asarray(alpha_coeff) / 2.0 * f0 * grid.c0 / (1e-2 * np_factor)
    return np.exp(-grid.dt * texp)


class MediumExponentialAttenuation:
    def __init__(self, grid, sound_speed, density, alpha_exp, beta, *, air_map=None) -> None:
        self.grid = grid
        self.is_3d = grid.is_3d
        self.sound_speed = np.atleast_2d(np.asarray(sound_speed, dtype=np.float64))
        self.density = np.atleast_2d(np.asarray(density, dtype=np.float64))
        self.alpha_exp = np.atleast_2d(np.asarray(alpha_exp, dtype=np.float64))
        self.beta = np.atleast_2d(np.asarray(beta, dtype=np.float64))
        self.air_map = (np.zeros_like(self.sound_speed, dtype=bool) if air_map is None
                        else np.asarray(air_map))

    @property
    def bulk_modulus(self):
        return np.multiply(self.sound_speed**2, self.density)

    @property
    def n_air(self) -> int:
        return int(np.asarray(self.air_map).sum())


def body_mask(shape, n_body: int) -> np.ndarray:
    """Normalised distance into the padding (0 inside, 1 at the outermost corner)."""
    r2 = 0.0
    for a, n in enumerate(shape):
        idx = np.arange(1, n + 1).reshape([-1 if b == a else 1 for b in range(len(shape))])
        r = np.where(idx <= n_body, n_body - idx + 1, np.where(idx > n - n_body, idx - (n - n_body), 0))
        r2 = r2 + r**2
    mask = np.sqrt(r2)
    if mask.max() > 0:
        mask = mask / mask.max()
    return mask


class PMLBuilderExponentialAttenuation:
    """Extended grid/medium/source/sensor for the exponential-attenuation engine."""

    def __init__(self, grid: Grid, sound_speed, density, alpha_coeff, beta, source: Source,
                 sensor: Sensor, *, air_map=None, m_spatial_order: int = N_TAPS,
                 n_pml_layer: int = 40) -> None:
        self.is_3d = grid.is_3d
        self.m_spatial_order = m_spatial_order
        self.n_pml_layer = n_pml_layer
        nb = self.num_boundary_points
        c = np.atleast_2d(np.asarray(sound_speed, dtype=np.float64))
        spacing = (grid.dx, grid.dy, grid.dz)
        domain = tuple((c.shape[k] + 2 * nb) * spacing[k] for k in range(c.ndim))
        self.extended_grid = Grid(domain_size=domain, f0=grid.f0, duration=grid.duration,
                                  c0=grid.c0, ppw=grid.ppw, cfl=grid.cfl)
        air = np.zeros_like(c, dtype=bool) if air_map is None else np.asarray(air_map)
        self.ext = {"c": extend_map(c, nb), "rho": extend_map(density, nb),
                    "alpha": extend_map(alpha_coeff, nb), "beta": extend_map(beta, nb),
                    "air": extend_map(air, nb)}
        self.extended_source = Source(source.p0, extend_map(source.mask, nb, fill_edge=False))
        self.extended_sensor = Sensor(extend_map(sensor.mask, nb, fill_edge=False),
                                      sampling_modulus_time=sensor.sampling_modulus_time)

    @property
    def num_boundary_points(self) -> int:
        return self.n_pml_layer + self.m_spatial_order

    def run(self, *, use_pml: bool = True) -> MediumExponentialAttenuation:
        e, g = self.ext, self.extended_grid
        a_exp = db_mhz_cm_to_a_exp(e["alpha"], g)
        if use_pml:
            a_exp = a_exp * (1 - body_mask(a_exp.shape, self.num_boundary_points))
        return MediumExponentialAttenuation(g, e["c"], e["rho"], a_exp, e["beta"], air_map=e["air"])
