"""Seeded synthetic workloads with the shapes, sizes and value distributions of the benchmark
configurations (no public dataset is involved; every medium is generated from a seed).

* ``plain_2d``: 2D forward, 768 (depth) x 512 (lateral) cells, dx = lambda/12 at 3 MHz,
  c0 = 1540 m/s, Courant 0.2, nt = 4000, PML 40 + transition 40 cells per side (extended grid
  944 x 688), background c 1540, rho 1000, alpha0 0.5, gamma 1.1; eight seeded random ellipses
  (semi-axes 1-5 mm) with c in [1450, 1650], rho in [900, 1100], alpha0 in [0, 1],
  gamma in [0.4, 1.6]; plane-wave source on depth row 0 (3 MHz, 2 cycles, 1 MPa); sensors on
  every cell of row 5, recorded every step.
* ``plain_3d`` (see :mod:`fullwave25_gb300.workloads3d`): 3D forward, 512^3 cells plus PML.

Relaxation parameters come from :func:`fullwave25_gb300.relaxation.default_table` (a stand-in
for the reference's missing lookup table).
"""

from __future__ import annotations

import numpy as np

from .grid import Grid
from .inputs import EngineInputs, build_inputs
from .medium import MediumRelaxationMaps
from .pml import PMLBuilder
from .pulse import gaussian_modulated_sinusoidal_signal
from .relaxation import default_table
from .source import Sensor, Source


def ellipse_medium_2d(shape, dx, seed: int = 0, n_ellipses: int = 8):
    """Background tissue plus ``n_ellipses`` seeded random ellipses; returns c, rho, a0, gamma."""
    rng = np.random.default_rng(seed)
    nx, ny = shape
    c = np.full(shape, 1540.0)
    rho = np.full(shape, 1000.0)
    a0 = np.full(shape, 0.5)
    gam = np.full(shape, 1.1)
    x = np.arange(nx)[:, None] * dx
    y = np.arange(ny)[None, :] * dx
    for _ in range(n_ellipses):
        cx, cy = rng.uniform(0, nx * dx), rng.uniform(0, ny * dx)
        ax, ay = rng.uniform(1e-3, 5e-3, size=2)
        th = rng.uniform(0, np.pi)
        u = (x - cx) * np.cos(th) + (y - cy) * np.sin(th)
        v = -(x - cx) * np.sin(th) + (y - cy) * np.cos(th)
        inside = (u / ax) ** 2 + (v / ay) ** 2 <= 1.0
        c[inside] = rng.uniform(1450, 1650)
        rho[inside] = rng.uniform(900, 1100)
        a0[inside] = rng.uniform(0, 1)
        gam[inside] = rng.uniform(0.4, 1.6)
    return c, rho, a0, gam


def plain_2d_problem(shape=(768, 512), nt: int = 4000, f0: float = 3e6, ppw: int = 12,
                     cfl: float = 0.2, n_pml: int = 40, n_transition: int = 40, seed: int = 0,
                     sensor_row: int = 5, p0: float = 1e6):
    """Grid, medium, source and sensor of the plain 2D forward workload (before PML padding)."""
    grid = Grid.from_cells(shape, f0=f0, nt=nt, ppw=ppw, cfl=cfl)
    c, rho, a0, gam = ellipse_medium_2d(shape, grid.dx, seed=seed)
    relax = default_table().lookup(a0, gam)
    medium = MediumRelaxationMaps(grid, c, rho, np.zeros(shape), relax)
    mask = np.zeros(shape, dtype=bool)
    mask[0, :] = True
    sig = gaussian_modulated_sinusoidal_signal(nt=nt, duration=grid.duration, ncycles=2,
                                               drop_off=2, f0=f0, p0=p0)
    source = Source(np.tile(sig, (int(mask.sum()), 1)), mask)
    smask = np.zeros(shape, dtype=bool)
    smask[sensor_row, :] = True
    sensor = Sensor(smask, sampling_modulus_time=1)
    return grid, medium, source, sensor, (n_pml, n_transition)


PHYSICS = ("isotropic", "aniso", "exp")


def plain_2d_inputs(physics: str = "isotropic", **kw) -> EngineInputs:
    """Engine inputs (PML-extended, 944 x 688 by default) of the plain 2D forward workload.

    ``physics``: "isotropic" (the two-mechanism relaxation engine), "aniso" (the same medium
    through the anisotropic-relaxation PML builder, one set of maps per derivative direction, as
    ``Solver(use_isotropic_relaxation=False)``), or "exp" (the exponential-attenuation engine
    with alpha0 of the same medium; its builder pads by PML + 8 cells only: 864 x 608)."""
    grid, medium, source, sensor, (n_pml, n_tr) = plain_2d_problem(**kw)
    if physics == "exp":
        from .exponential import PMLBuilderExponentialAttenuation  # noqa: PLC0415
        from .inputs import build_inputs_exponential  # noqa: PLC0415

        c, rho, a0, _ = ellipse_medium_2d(grid.shape, grid.dx, seed=kw.get("seed", 0))
        b = PMLBuilderExponentialAttenuation(grid, c, rho, a0, np.zeros(grid.shape), source,
                                             sensor, n_pml_layer=n_pml)
        return build_inputs_exponential(b.extended_grid, b.run(), b.extended_source,
                                        b.extended_sensor)
    if physics not in PHYSICS:
        raise ValueError(f"unknown physics {physics!r}")
    iso = physics == "isotropic"
    medium.use_isotropic_relaxation = iso   # as the solver sets it before building
    b = PMLBuilder(grid, medium, source, sensor, n_pml_layer=n_pml, n_transition_layer=n_tr,
                   use_isotropic_relaxation=iso)
    return build_inputs(b.extended_grid, b.run(), b.extended_source, b.extended_sensor)


def algorithmic_bytes_per_cell(ndim: int, beta: bool = False, physics: str = "isotropic") -> int:
    """Algorithmic HBM bytes of one cell-update: 4 * (2 S + M).

    Isotropic engine: S state fields read and written once per step (p, ndim velocities, 2 ndim
    gradient and 2 ndim divergence memory variables) and M = 12 read-only maps read once per
    step, the figure of the workload definition (rho, K, kappau, kappax, four a/b pairs and the
    tap index; plus beta when it is not zero): 136 B in 2D, 176 B in 3D. Anisotropic engine: 10
    more maps per further axis (kappa, two a/b pairs for each derivative direction): 176 B in
    2D, 256 B in 3D. Exponential engine: S = p and the velocities, M = rho, K, a_exp and the tap
    index: 40 B in 2D, 48 B in 3D.
    """
    if physics == "exp":
        return 4 * (2 * (1 + ndim) + 4 + (1 if beta else 0))
    s = 1 + ndim + 4 * ndim
    m = 12 + (1 if beta else 0) + (10 * (ndim - 1) if physics == "aniso" else 0)
    return 4 * (2 * s + m)
