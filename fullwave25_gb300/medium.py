"""Relaxation medium maps and their recursive-convolution coefficients.

Mirrors ``fullwave/medium.py:20-406`` (``MediumRelaxationMaps``): the ten relaxation parameter
maps per cell (``kappa_x1, kappa_x2`` and, per mechanism ``nu``, ``d_x{1,2}_nu`` and
``alpha_x{1,2}_nu``), the per-cell sort of mechanisms by time constant ``d/kappa + alpha``
(medium.py:121-209), the bulk modulus ``K = c^2 rho`` (:255-258) and the memory-variable
coefficients

    b = exp(-(d/kappa + alpha) * dT)
    a = d / (kappa * (d + kappa * alpha) + 1e-10) * (b - 1)          (medium.py:273-289)

with the engine's names: ``u`` is the pressure-gradient operator (nabla_1, parameters ``x1``)
and ``x`` the velocity-divergence operator (nabla_2, parameters ``x2``) (medium.py:357-372).
"""

from __future__ import annotations

import numpy as np

RELAXATION_KEYS_ORDER = ("kappa_x1", "kappa_x2")


def relaxation_param_keys(n_relaxation_mechanisms: int = 2) -> list:
    """Parameter names in the reference's order (fullwave/solver/utils.py:68-86)."""
    keys = ["kappa_x1", "kappa_x2"]
    for nu in range(1, n_relaxation_mechanisms + 1):
        keys += [f"d_x1_nu{nu}", f"alpha_x1_nu{nu}", f"d_x2_nu{nu}", f"alpha_x2_nu{nu}"]
    return keys


def calc_a_and_b(d, kappa, alpha, dt):
    """Recursive-convolution coefficients ``(a, b)`` of one relaxation mechanism."""
    d = np.asarray(d, dtype=np.float64)
    kappa = np.asarray(kappa, dtype=np.float64)
    alpha = np.asarray(alpha, dtype=np.float64)
    b = np.exp(-(d / kappa + alpha) * dt)
    a = d / (kappa * (d + kappa * alpha) + 1e-10) * (b - 1)
    return a, b


class MediumRelaxationMaps:
    """Medium given directly by relaxation parameter maps (the engine's physical input)."""

    def __init__(self, grid, sound_speed, density, beta, relaxation_param_dict, *,
                 air_map=None, n_relaxation_mechanisms: int = 2,
                 use_isotropic_relaxation: bool = True) -> None:
        if n_relaxation_mechanisms != 2:
            raise ValueError("Only n_relaxation_mechanisms=2 are supported currently.")
        self.grid = grid
        self.is_3d = grid.is_3d
        self.n_relaxation_mechanisms = n_relaxation_mechanisms
        self.sound_speed = np.atleast_2d(np.asarray(sound_speed, dtype=np.float64))
        self.density = np.atleast_2d(np.asarray(density, dtype=np.float64))
        self.beta = np.atleast_2d(np.asarray(beta, dtype=np.float64))
        self.air_map = (np.zeros_like(self.sound_speed, dtype=bool) if air_map is None
                        else np.asarray(air_map))
        self.relaxation_param_dict = self._sorted_params(relaxation_param_dict)
        self.use_isotropic_relaxation = use_isotropic_relaxation
        self.relaxation_param_dict_for_fw2 = self.calc_relaxation_param_dict_for_fw2(
            use_isotropic_relaxation=use_isotropic_relaxation)

    # -- parameters -------------------------------------------------------------------------
    def _sorted_params(self, params: dict) -> dict:
        keys = relaxation_param_keys(self.n_relaxation_mechanisms)
        if set(params) != set(keys):
            raise ValueError(f"Unknown relaxation parameter keys: {set(params) ^ set(keys)}")
        for v in params.values():
            if np.shape(v) != self.sound_speed.shape:
                raise ValueError("Relaxation parameter map shape error: "
                                 f"{np.shape(v)} != {self.sound_speed.shape} (domain shape)")
        out = {"kappa_x1": np.atleast_2d(params["kappa_x1"]),
               "kappa_x2": np.atleast_2d(params["kappa_x2"])}
        nus = range(1, self.n_relaxation_mechanisms + 1)
        for op in ("x1", "x2"):
            kappa = params[f"kappa_{op}"]
            d = np.stack([params[f"d_{op}_nu{nu}"] for nu in nus], axis=-1)
            alpha = np.stack([params[f"alpha_{op}_nu{nu}"] for nu in nus], axis=-1)
            tau = d / np.asarray(kappa)[..., None] + alpha
            order = np.argsort(tau, axis=-1)
            d = np.take_along_axis(d, order, axis=-1)
            alpha = np.take_along_axis(alpha, order, axis=-1)
            for nu in nus:
                out[f"d_{op}_nu{nu}"] = np.atleast_2d(d[..., nu - 1])
                out[f"alpha_{op}_nu{nu}"] = np.atleast_2d(alpha[..., nu - 1])
        return {k: out[k] for k in keys}

    @property
    def bulk_modulus(self) -> np.ndarray:
        return np.multiply(self.sound_speed**2, self.density)

    @property
    def n_air(self) -> int:
        return int(np.asarray(self.air_map).sum())

    n_coords_zero = n_air

    def relaxation_coefficients(self) -> dict:
        """``kappa_x{1,2}`` and ``a/b_pml_x{1,2}_nu{nu}`` per cell (medium.py:292-330)."""
        p = self.relaxation_param_dict
        out = {"kappa_x1": p["kappa_x1"], "kappa_x2": p["kappa_x2"]}
        for nu in range(1, self.n_relaxation_mechanisms + 1):
            for op in ("x1", "x2"):
                out[f"a_pml_{op}_nu{nu}"], out[f"b_pml_{op}_nu{nu}"] = calc_a_and_b(
                    p[f"d_{op}_nu{nu}"], p[f"kappa_{op}"], p[f"alpha_{op}_nu{nu}"], self.grid.dt)
        return out

    def calc_relaxation_param_dict_for_fw2(self, *, use_isotropic_relaxation: bool = True) -> dict:
        """Coefficient maps under the engine's names (medium.py:332-406)."""
        axes_u = ["u"] if use_isotropic_relaxation else (["u", "w", "v"] if self.is_3d else ["u", "w"])
        axes_x = ["x"] if use_isotropic_relaxation else (["x", "y", "z"] if self.is_3d else ["x", "y"])
        coef = self.relaxation_coefficients()
        out = {}
        for ax in axes_x:
            out[f"kappa_{ax}"] = coef["kappa_x2"].copy()
        for ax in axes_u:
            out[f"kappa_{ax}"] = coef["kappa_x1"].copy()
        for nu in range(1, self.n_relaxation_mechanisms + 1):
            for ax in axes_u:
                out[f"a_pml_{ax}{nu}"] = coef[f"a_pml_x1_nu{nu}"].copy()
                out[f"b_pml_{ax}{nu}"] = coef[f"b_pml_x1_nu{nu}"].copy()
            for ax in axes_x:
                out[f"a_pml_{ax}{nu}"] = coef[f"a_pml_x2_nu{nu}"].copy()
                out[f"b_pml_{ax}{nu}"] = coef[f"b_pml_x2_nu{nu}"].copy()
        return out

    def build(self) -> "MediumRelaxationMaps":
        return self


class Medium:
    """Medium given by attenuation maps (mirrors ``fullwave/medium.py:753-1156``).

    ``build()`` maps (alpha0, gamma) to relaxation parameters by table lookup
    (:class:`fullwave25_gb300.relaxation.RelaxationTable`; the reference's ``.mat`` table when
    one is given, else the stand-in table) and returns a :class:`MediumRelaxationMaps`;
    ``build_exponential()`` returns the exponential-attenuation medium (medium.py:1068-1111).
    """

    def __init__(self, grid, sound_speed, density, alpha_coeff, alpha_power, beta, *,
                 air_map=None, relaxation_table=None, n_relaxation_mechanisms: int = 2,
                 use_isotropic_relaxation: bool = True) -> None:
        if n_relaxation_mechanisms != 2:
            raise ValueError("Only n_relaxation_mechanisms=2 are supported currently.")
        self.grid = grid
        self.is_3d = grid.is_3d
        self.sound_speed = np.atleast_2d(np.asarray(sound_speed, dtype=np.float64))
        self.density = np.atleast_2d(np.asarray(density, dtype=np.float64))
        self.alpha_coeff = np.atleast_2d(np.asarray(alpha_coeff, dtype=np.float64))
        self.alpha_power = np.atleast_2d(np.asarray(alpha_power, dtype=np.float64))
        self.beta = np.atleast_2d(np.asarray(beta, dtype=np.float64))
        self.air_map = (np.zeros_like(self.sound_speed, dtype=bool) if air_map is None
                        else np.asarray(air_map))
        self.relaxation_table = relaxation_table
        self.n_relaxation_mechanisms = n_relaxation_mechanisms
        self.use_isotropic_relaxation = use_isotropic_relaxation

    @property
    def bulk_modulus(self):
        return np.multiply(self.sound_speed**2, self.density)

    def build(self) -> MediumRelaxationMaps:
        from .relaxation import default_table  # noqa: PLC0415

        table = self.relaxation_table or default_table()
        params = table.lookup(self.alpha_coeff, self.alpha_power)
        return MediumRelaxationMaps(self.grid, self.sound_speed, self.density, self.beta, params,
                                    air_map=self.air_map,
                                    use_isotropic_relaxation=self.use_isotropic_relaxation)

    def build_exponential(self):
        from .exponential import MediumExponentialAttenuation, db_mhz_cm_to_a_exp  # noqa: PLC0415

        return MediumExponentialAttenuation(self.grid, self.sound_speed, self.density,
                                            db_mhz_cm_to_a_exp(self.alpha_coeff, self.grid),
                                            self.beta, air_map=self.air_map)
