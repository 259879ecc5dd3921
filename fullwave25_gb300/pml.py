"""Grid extension and relaxing PML for the engine's coefficient maps.

Restates ``fullwave/solver/pml_builder.py`` for the isotropic and anisotropic relaxation maps:

* every map is padded by ``n_transition + n_pml + 8`` cells per side, replicating edge values
  for material maps and zero-filling masks (pml_builder.py:270-276, :321-704);
* the relaxation parameters are ramped towards PML targets, one axis after the other
  (pml_builder.py:842-1254, :1256-1498): mechanism 1 gets ``d -> d_target`` with a quadratic
  ramp and ``alpha -> 0`` with a linear ramp over the PML + transition layers; mechanisms >= 2 get
  ``d, alpha -> 0`` with a cosine ramp inside the transition layer;
  ``d_target = -(n+1) c0 ln(R) / (2 (L_pml + L_transition))`` with ``n = 2``, ``R = 1e-30``
  (Komatitsch & Martin 2007, as cited at pml_builder.py:850-885);
* ``a/b`` are recomputed from the ramped parameters (pml_builder.py:794-810).
"""

from __future__ import annotations

import numpy as np

from .coefficients import N_TAPS
from .grid import Grid
from .medium import MediumRelaxationMaps, calc_a_and_b
from .source import Sensor, Source


def extend_map(arr: np.ndarray, n_boundary: int, *, fill_edge: bool = True) -> np.ndarray:
    """Pad every axis by ``n_boundary`` cells: edge replication, or zeros for masks."""
    arr = np.asarray(arr)
    if fill_edge:
        return np.pad(arr.astype(np.float64), n_boundary, mode="edge")
    return np.pad(arr.astype(np.float64), n_boundary, mode="constant", constant_values=0)


def _transition(kind: str, n: int, n_polynomial: float) -> np.ndarray:
    x = np.linspace(0, 1, n + 1)
    if kind == "linear":
        return x
    if kind == "polynomial":
        return x**n_polynomial
    if kind == "cosine":
        return 0.5 * (1 - np.cos(np.pi * x))
    if kind == "smooth":
        def part(v):
            return np.where(v > 0, np.exp(-1 / (v + 1e-20)), 0)
        return part(x) / (part(x) + part(1 - x))
    raise ValueError(f"Invalid transition type: {kind}.")


def ramp_axis(arr: np.ndarray, target: float, axis: int, *, thickness: int, offset: int,
              kind: str, n_polynomial: float = 2, ghost: int = N_TAPS) -> np.ndarray:
    """Ramp ``arr`` towards ``target`` at both ends of ``axis`` (pml_builder.py:1256-1498).

    The outermost ``ghost + offset`` cells are set to ``target``; the next ``thickness + 1``
    cells blend from ``target`` to the first interior value with the transition function.
    """
    out = np.moveaxis(arr, axis, 0)  # view: writes land in arr
    n = out.shape[0]
    tf = _transition(kind, thickness, n_polynomial)
    shape = (-1,) + (1,) * (out.ndim - 1)
    out[: ghost + offset + thickness] = target
    out[n - ghost - thickness - offset:] = target
    up_start, up_end = ghost + offset - 1, ghost + offset + thickness
    down_start, down_end = n - ghost - thickness - offset - 1, n - ghost - offset
    up_vals = out[up_end][None].copy()
    down_vals = out[down_start][None].copy()
    out[up_start:up_end] = up_vals - tf[::-1].reshape(shape) * (up_vals - target)
    out[down_start:down_end] = down_vals - tf.reshape(shape) * (down_vals - target)
    return arr


class PMLBuilder:
    """Extended grid, medium, source and sensor with the relaxing PML applied.

    Mirrors ``fullwave.solver.pml_builder.PMLBuilder`` (constructor at pml_builder.py:114-267,
    ``run`` at :812-840) for a :class:`MediumRelaxationMaps` input.
    """

    def __init__(self, grid: Grid, medium: MediumRelaxationMaps, source: Source, sensor: Sensor,
                 *, m_spatial_order: int = N_TAPS, n_pml_layer: int = 40,
                 n_transition_layer: int = 40, use_isotropic_relaxation: bool = True) -> None:
        self.grid_org, self.medium_org = grid, medium
        self.source_org, self.sensor_org = source, sensor
        self.is_3d = grid.is_3d
        self.use_isotropic_relaxation = use_isotropic_relaxation
        self.m_spatial_order = m_spatial_order
        self.n_pml_layer = n_pml_layer
        self.n_transition_layer = n_transition_layer
        nb = self.num_boundary_points
        spacing = (grid.dx, grid.dy, grid.dz)
        domain = tuple((medium.sound_speed.shape[k] + 2 * nb) * spacing[k]
                       for k in range(medium.sound_speed.ndim))
        self.extended_grid = Grid(domain_size=domain, f0=grid.f0, duration=grid.duration,
                                  c0=grid.c0, ppw=grid.ppw, cfl=grid.cfl)
        self.extended_medium = MediumRelaxationMaps(
            grid=self.extended_grid,
            sound_speed=extend_map(medium.sound_speed, nb),
            density=extend_map(medium.density, nb),
            beta=extend_map(medium.beta, nb),
            relaxation_param_dict={k: extend_map(v, nb)
                                   for k, v in medium.relaxation_param_dict.items()},
            air_map=extend_map(medium.air_map, nb, fill_edge=False),
            n_relaxation_mechanisms=medium.n_relaxation_mechanisms,
        )
        self.extended_source = Source(source.p0, extend_map(source.mask, nb, fill_edge=False))
        self.extended_sensor = Sensor(extend_map(sensor.mask, nb, fill_edge=False),
                                      sampling_modulus_time=sensor.sampling_modulus_time)
        self.pml_layer_m = self.extended_grid.dx * n_pml_layer
        self.transition_layer_m = self.extended_grid.dx * n_transition_layer
        self.n_polynomial = 2
        self.theoritical_reflection_coefficient = 1e-30
        if self.n_pml_layer == 0:
            self.n_transition_layer = 0

    @property
    def num_boundary_points(self) -> int:
        return self.n_transition_layer + self.n_pml_layer + self.m_spatial_order

    @property
    def d_target_pml(self) -> float:
        return (-(self.n_polynomial + 1) * self.extended_grid.c0
                * np.log(self.theoritical_reflection_coefficient)
                / (2 * (self.pml_layer_m + self.transition_layer_m)))

    def run(self, *, use_pml: bool = True) -> MediumRelaxationMaps:
        medium = self.extended_medium.build()
        if not use_pml:
            return medium
        return self._apply_pml(medium)

    def _apply_pml(self, medium: MediumRelaxationMaps) -> MediumRelaxationMaps:
        ndim = 3 if self.is_3d else 2
        params = medium.relaxation_param_dict
        if self.use_isotropic_relaxation:
            ops = {"u": "x1", "x": "x2"}
        elif self.is_3d:
            ops = {"u": "x1", "w": "x1", "v": "x1", "x": "x2", "y": "x2", "z": "x2"}
        else:
            ops = {"u": "x1", "w": "x1", "x": "x2", "y": "x2"}
        npml, ntr = self.n_pml_layer, self.n_transition_layer
        out = {}
        for ax, op in ops.items():
            out[f"kappa_{ax}"] = params[f"kappa_{op}"].copy()
            for nu in range(1, medium.n_relaxation_mechanisms + 1):
                for var in ("alpha", "d"):
                    arr = params[f"{var}_{op}_nu{nu}"].copy()
                    for axis in range(ndim):
                        if nu == 1:
                            target = 0.0 if var == "alpha" else self.d_target_pml
                            kind = "linear" if var == "alpha" else "polynomial"
                            arr = ramp_axis(arr, target, axis, thickness=npml + ntr, offset=0,
                                            kind=kind, n_polynomial=self.n_polynomial,
                                            ghost=self.m_spatial_order)
                        else:
                            if ntr == 0:
                                raise ValueError("Transition layer is not defined. Set "
                                                 "transit_within_transition_layer to False or "
                                                 "define n_transition_layer.")
                            arr = ramp_axis(arr, 0.0, axis, thickness=ntr, offset=npml,
                                            kind="cosine", ghost=self.m_spatial_order)
                    out[f"{var}_{ax}_nu{nu}"] = arr
        for nu in range(1, medium.n_relaxation_mechanisms + 1):
            for ax in ops:
                out[f"a_pml_{ax}{nu}"], out[f"b_pml_{ax}{nu}"] = calc_a_and_b(
                    out[f"d_{ax}_nu{nu}"], out[f"kappa_{ax}"], out[f"alpha_{ax}_nu{nu}"],
                    medium.grid.dt)
        medium.relaxation_param_dict_for_fw2.update(out)
        return medium
