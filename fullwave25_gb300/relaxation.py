"""Attenuation (alpha0, gamma) -> two-mechanism relaxation parameters by table lookup.

Lookup semantics follow ``fullwave/utils/relaxation_parameters.py:18-242``: the table has shape
``[n_alpha, n_power, 10]`` with columns in the order ``kappa_x1, kappa_x2`` then, per mechanism,
``d_x1, alpha_x1, d_x2, alpha_x2`` (fullwave/solver/utils.py:68-86); inputs are clipped to the
table range and mapped to bins with ``searchsorted`` on the bin lists rounded to 10 digits.
A table in the reference's ``.mat`` format (keys ``database``, ``alpha_0_list``, ``power_list``,
``invalid_matrix``) can be loaded with :meth:`RelaxationTable.from_mat`.

The reference's own table file is not part of its source checkout, so this module can also build
a stand-in table: for every (alpha0, gamma) bin it fits the attenuation of the stretched
coordinate ``s(w) = 1 + sum_nu d_nu / (alpha_nu + i w)`` (the same relaxation form the engine
integrates) to the power law ``alpha0 f^gamma`` over 0.5-10 MHz with two mechanisms, choosing
the relaxation rates from a fixed candidate set and the strengths by non-negative least squares.
It is a plausible physical parameter set for synthetic workloads, not the reference's table.
"""

from __future__ import annotations

import itertools
from dataclasses import dataclass

import numpy as np

from .medium import relaxation_param_keys

NP_PER_DB = 1.0 / 8.685889638065037


@dataclass
class RelaxationTable:
    table: np.ndarray          # [n_alpha, n_power, 10]
    alpha_list: np.ndarray     # [n_alpha]
    power_list: np.ndarray     # [n_power]
    invalid: np.ndarray        # [n_alpha, n_power] bool

    @classmethod
    def from_mat(cls, path) -> "RelaxationTable":
        from scipy.io import loadmat  # noqa: PLC0415

        db = loadmat(path)
        return cls(np.asarray(db["database"]), np.asarray(db["alpha_0_list"]).ravel(),
                   np.asarray(db["power_list"]).ravel(),
                   np.asarray(db["invalid_matrix"]).astype(bool))

    def lookup(self, alpha_coeff, alpha_power) -> dict:
        """Per-cell parameter maps for ``alpha_coeff`` [dB/MHz^gamma/cm] and ``alpha_power``."""
        a = np.clip(np.asarray(alpha_coeff, dtype=np.float64), self.alpha_list.min(),
                    self.alpha_list.max())
        g = np.clip(np.asarray(alpha_power, dtype=np.float64), self.power_list.min(),
                    self.power_list.max().round(4))
        ia = np.clip(np.searchsorted(self.alpha_list.round(10), a), 0, len(self.alpha_list) - 1)
        ig = np.clip(np.searchsorted(self.power_list.round(10), g), 0, len(self.power_list) - 1)
        out = self.table[ia, ig, :]
        return {k: out[..., i] for i, k in enumerate(relaxation_param_keys(2))}


def _fit_bin(target, basis, pairs):
    """Best two-mechanism non-negative fit of ``target`` [n_f] over candidate rate pairs."""
    best = (np.inf, None, None)
    for (i, j) in pairs:
        A = np.stack([basis[i], basis[j]], axis=1)
        coef, *_ = np.linalg.lstsq(A, target, rcond=None)
        if (coef < 0).any():  # project onto the non-negative orthant (one-sided fits)
            cands = []
            for k in (0, 1):
                col = A[:, k]
                ck = max(float(col @ target) / float(col @ col), 0.0)
                c = np.zeros(2)
                c[k] = ck
                cands.append(c)
            coef = min(cands, key=lambda c: np.linalg.norm(A @ c - target))
        err = np.linalg.norm(A @ coef - target)
        if err < best[0]:
            best = (err, (i, j), coef)
    return best


def synthetic_table(alpha_list=None, power_list=None, c0: float = 1540.0) -> RelaxationTable:
    """Stand-in lookup table fitted as described in the module docstring."""
    alpha_list = np.linspace(0.0, 1.5, 31) if alpha_list is None else np.asarray(alpha_list)
    power_list = np.linspace(0.4, 1.6, 25) if power_list is None else np.asarray(power_list)
    f = np.geomspace(0.5e6, 10e6, 24)
    w = 2 * np.pi * f
    rates = 2 * np.pi * np.geomspace(0.2e6, 50e6, 10)
    # attenuation [Np/m] of one mechanism with unit strength: (w/c) * Im(1/s) ~ w^2/(c(r^2+w^2))
    basis = np.stack([w**2 / (c0 * (r**2 + w**2)) for r in rates])
    pairs = list(itertools.combinations(range(len(rates)), 2))
    table = np.zeros((len(alpha_list), len(power_list), 10))
    invalid = np.zeros((len(alpha_list), len(power_list)), dtype=bool)
    for ia, a0 in enumerate(alpha_list):
        for ig, gam in enumerate(power_list):
            target = a0 * (f / 1e6) ** gam * 100.0 * NP_PER_DB
            row = np.zeros(10)
            row[0] = row[1] = 1.0
            if a0 > 0:
                _, (i, j), coef = _fit_bin(target, basis, pairs)
                for nu, (r, dnu) in enumerate(((rates[i], coef[0]), (rates[j], coef[1]))):
                    base = 2 + 4 * nu
                    row[base + 0] = dnu        # d_x1_nu
                    row[base + 1] = r          # alpha_x1_nu
                    row[base + 2] = dnu        # d_x2_nu
                    row[base + 3] = r          # alpha_x2_nu
            else:
                for nu in range(2):
                    row[2 + 4 * nu + 1] = row[2 + 4 * nu + 3] = rates[nu]
            table[ia, ig] = row
    return RelaxationTable(table, alpha_list, power_list, invalid)


_DEFAULT = None


def default_table() -> RelaxationTable:
    global _DEFAULT
    if _DEFAULT is None:
        _DEFAULT = synthetic_table()
    return _DEFAULT
