"""The FP64 NumPy adjoint against central finite differences of the FP64 oracle."""

import numpy as np
import pytest

from fdtd_adjoint import (EXP_GRAD_KEYS, GRAD_KEYS, GRAD_LETTERS, AdjointOracle, aniso_grad_keys,
                          misfit, misfit_and_gradient)
from fdtd_oracle import GHOST, Oracle
from golden_io import load_case_inputs


def _small(name, nt):
    inp = load_case_inputs(name)
    inp.nt = nt
    inp.icmat = np.ascontiguousarray(inp.icmat[:, :nt])
    return inp


@pytest.fixture(scope="module")
def case():
    inp = _small("2d_small", 70)
    # observed data: the same experiment with a slightly different medium
    obs_inp = _small("2d_small", 70)
    obs_inp.maps = dict(obs_inp.maps)
    obs_inp.maps["K"] = (obs_inp.maps["K"] * np.float32(1.02)).astype(np.float32)
    observed = Oracle(obs_inp).run()
    J, G, traces = misfit_and_gradient(inp, observed)
    return inp, observed, J, G


def _base_map(o, key):
    return {"rdt_rho": o.rdt_rho, "dt_k": o.dt_k, "inv_ku": o.inv_kappa_u,
            "inv_kx": o.inv_kappa_x}.get(key) if key in ("rdt_rho", "dt_k", "inv_ku", "inv_kx") \
        else getattr(o, key[:2])[int(key[2]) - 1]


@pytest.mark.parametrize("key", GRAD_KEYS)
def test_gradient_matches_central_differences(case, key):
    inp, observed, J, G = case
    o = Oracle(inp)
    base = _base_map(o, key)
    rng = np.random.default_rng(sum(map(ord, key)))
    # cells near the source/sensor rows and in the medium interior
    cells = [(int(rng.integers(2, base.shape[0] - 2)), int(rng.integers(2, base.shape[1] - 2)))
             for _ in range(3)]
    for c in cells:
        mag = abs(base[c]) if base[c] != 0 else float(np.abs(base).mean())
        h = 1e-4 * mag
        plus, minus = base.copy(), base.copy()
        plus[c] += h
        minus[c] -= h
        fd = (misfit(inp, observed, {key: plus}) - misfit(inp, observed, {key: minus})) / (2 * h)
        ad = G[key][c]
        # central differences of an FP64 quadratic: agreement to ~1e-6 relative, with an
        # absolute floor for cells the traces barely depend on
        floor = 1e-10 * abs(J) / mag
        assert abs(fd - ad) <= 1e-5 * max(abs(fd), abs(ad)) + floor, \
            f"{key} at {c}: adjoint {ad:.6e} vs finite difference {fd:.6e}"


def test_gradient_is_nonzero_and_finite(case):
    inp, observed, J, G = case
    assert J > 0
    for k in GRAD_KEYS:
        assert np.isfinite(G[k]).all()
    assert np.abs(G["dt_k"]).max() > 0 and np.abs(G["rdt_rho"]).max() > 0


@pytest.fixture(scope="module")
def exp_case():
    inp = _small("2d_exp", 70)
    obs_inp = _small("2d_exp", 70)
    obs_inp.maps = dict(obs_inp.maps)
    obs_inp.maps["K"] = (obs_inp.maps["K"] * np.float32(1.02)).astype(np.float32)
    observed = Oracle(obs_inp).run()
    J, G, traces = misfit_and_gradient(inp, observed)
    return inp, observed, J, G


@pytest.mark.parametrize("key", EXP_GRAD_KEYS)
def test_exponential_gradient_matches_central_differences(exp_case, key):
    """The exponential-attenuation engine's adjoint (gradients with respect to dt/rho, dt*K and
    a_exp) against central differences of the FP64 oracle, same bounds as above."""
    inp, observed, J, G = exp_case
    o = Oracle(inp)
    base = getattr(o, key)
    assert np.isfinite(G[key]).all() and np.abs(G[key]).max() > 0
    rng = np.random.default_rng(sum(map(ord, key)))
    cells = [(int(rng.integers(2, base.shape[0] - 2)), int(rng.integers(2, base.shape[1] - 2)))
             for _ in range(3)]
    for c in cells:
        mag = abs(base[c]) if base[c] != 0 else float(np.abs(base).mean())
        h = 1e-4 * mag
        plus, minus = base.copy(), base.copy()
        plus[c] += h
        minus[c] -= h
        fd = (misfit(inp, observed, {key: plus}) - misfit(inp, observed, {key: minus})) / (2 * h)
        ad = G[key][c]
        floor = 1e-10 * abs(J) / mag
        assert abs(fd - ad) <= 1e-5 * max(abs(fd), abs(ad)) + floor, \
            f"{key} at {c}: adjoint {ad:.6e} vs finite difference {fd:.6e}"


@pytest.fixture(scope="module")
def aniso_case():
    inp = _small("2d_aniso", 70)
    obs_inp = _small("2d_aniso", 70)
    obs_inp.maps = dict(obs_inp.maps)
    obs_inp.maps["K"] = (obs_inp.maps["K"] * np.float32(1.02)).astype(np.float32)
    observed = Oracle(obs_inp).run()
    J, G, traces = misfit_and_gradient(inp, observed)
    return inp, observed, J, G


def _aniso_base(o, key):
    if key in ("rdt_rho", "dt_k"):
        return getattr(o, key)
    letter = key[5] if key.startswith("inv_k") else key[1]
    side = 0 if letter in GRAD_LETTERS[0] else 1
    ik, aa, bb = (o.axis_u if side == 0 else o.axis_x)[GRAD_LETTERS[side].index(letter)]
    if key.startswith("inv_k"):
        return ik
    return (aa if key[0] == "a" else bb)[int(key[2]) - 1]


@pytest.mark.parametrize("key", aniso_grad_keys(2))
def test_anisotropic_gradient_matches_central_differences(aniso_case, key):
    """The anisotropic engine's adjoint (one map set per derivative axis: 22 gradients in 2D)
    against central differences of the FP64 oracle, same bounds as above."""
    inp, observed, J, G = aniso_case
    base = _aniso_base(Oracle(inp), key)
    assert np.isfinite(G[key]).all() and np.abs(G[key]).max() > 0
    rng = np.random.default_rng(sum(map(ord, key)))
    cells = [(int(rng.integers(2, base.shape[0] - 2)), int(rng.integers(2, base.shape[1] - 2)))
             for _ in range(2)]
    for c in cells:
        mag = abs(base[c]) if base[c] != 0 else float(np.abs(base).mean())
        h = 1e-4 * mag
        plus, minus = base.copy(), base.copy()
        plus[c] += h
        minus[c] -= h
        fd = (misfit(inp, observed, {key: plus}) - misfit(inp, observed, {key: minus})) / (2 * h)
        ad = G[key][c]
        floor = 1e-10 * abs(J) / mag
        assert abs(fd - ad) <= 1e-5 * max(abs(fd), abs(ad)) + floor, \
            f"{key} at {c}: adjoint {ad:.6e} vs finite difference {fd:.6e}"


def _beta_case(name, nt, beta=None):
    inp = _small(name, nt)
    if beta is not None:   # a nonlinear variant of a linear golden case
        inp.maps = dict(inp.maps)
        inp.maps["beta"] = np.full(inp.shape, beta, dtype=np.float32)
    obs_inp = _small(name, nt)
    obs_inp.maps = dict(inp.maps)
    obs_inp.maps["K"] = (obs_inp.maps["K"] * np.float32(1.02)).astype(np.float32)
    observed = Oracle(obs_inp).run()
    J, G, traces = misfit_and_gradient(inp, observed)
    return inp, observed, J, G


@pytest.fixture(scope="module")
def beta_cases():
    return {"relaxation": _beta_case("2d_air_beta", 70),
            "exponential": _beta_case("2d_exp", 70, beta=8.0)}


@pytest.mark.parametrize("engine,key", [("relaxation", k) for k in GRAD_KEYS + ("beta2dt",)] +
                         [("exponential", k) for k in EXP_GRAD_KEYS + ("beta2dt",)])
def test_nonlinear_gradient_matches_central_differences(beta_cases, engine, key):
    """The adjoint of the nonlinear engines (beta != 0: the coefficient of the divergence is
    dt K + 2 dt beta p, so the pressure adjoint is linearised around the stored forward states)
    against central differences of the FP64 oracle, including the gradient with respect to
    2 dt beta; the relaxation case also has air cells and a recording interval above 1."""
    inp, observed, J, G = beta_cases[engine]
    o = Oracle(inp)
    assert o.has_beta
    base = _base_map(o, key) if engine == "relaxation" and key != "beta2dt" else getattr(o, key)
    assert np.isfinite(G[key]).all() and np.abs(G[key]).max() > 0
    rng = np.random.default_rng(sum(map(ord, key)) + len(engine))
    cells = [(int(rng.integers(2, base.shape[0] - 2)), int(rng.integers(2, base.shape[1] - 2)))
             for _ in range(2)]
    for c in cells:
        mag = abs(base[c]) if base[c] != 0 else float(np.abs(base).mean())
        h = 1e-4 * mag
        plus, minus = base.copy(), base.copy()
        plus[c] += h
        minus[c] -= h
        fd = (misfit(inp, observed, {key: plus}) - misfit(inp, observed, {key: minus})) / (2 * h)
        ad = G[key][c]
        floor = 1e-10 * abs(J) / mag
        assert abs(fd - ad) <= 1e-5 * max(abs(fd), abs(ad)) + floor, \
            f"{engine} {key} at {c}: adjoint {ad:.6e} vs finite difference {fd:.6e}"


@pytest.mark.parametrize("name,beta,keys", [
    ("3d_small", None, ("rdt_rho", "dt_k", "inv_ku", "bx2")),
    ("3d_aniso", 6.0, ("inv_kv", "az1", "bw2", "beta2dt")),
    ("3d_exp", 8.0, ("rdt_rho", "dt_k", "a_exp", "beta2dt")),
])
def test_3d_gradients_match_central_differences(name, beta, keys):
    """The FP64 adjoint in 3D (isotropic, anisotropic with beta, exponential with beta) against
    central differences of the FP64 oracle on a short run of the golden 3D cases."""
    inp = _small(name, 16)
    if beta is not None:
        inp.maps = dict(inp.maps)
        inp.maps["beta"] = np.full(inp.shape, beta, dtype=np.float32)
    obs_inp = _small(name, 16)
    obs_inp.maps = dict(inp.maps)
    obs_inp.maps["K"] = (obs_inp.maps["K"] * np.float32(1.02)).astype(np.float32)
    observed = Oracle(obs_inp).run()
    J, G, _ = misfit_and_gradient(inp, observed)
    o = Oracle(inp)
    for key in keys:
        if key in ("rdt_rho", "dt_k", "a_exp", "beta2dt"):
            base = getattr(o, key)
        elif o.axis_u[0] is not None:
            base = _aniso_base(o, key)
        else:
            base = _base_map(o, key)
        assert np.abs(G[key]).max() > 0, key
        # the cell where this gradient is largest: well above the differences' rounding
        c = np.unravel_index(int(np.argmax(np.abs(G[key]))), G[key].shape)
        mag = abs(base[c]) if base[c] != 0 else float(np.abs(base).mean())
        h = 1e-4 * mag
        plus, minus = base.copy(), base.copy()
        plus[c] += h
        minus[c] -= h
        fd = (misfit(inp, observed, {key: plus}) - misfit(inp, observed, {key: minus})) / (2 * h)
        ad = G[key][c]
        assert abs(fd - ad) <= 1e-5 * max(abs(fd), abs(ad)) + 1e-10 * abs(J) / mag, \
            f"{name} {key} at {c}: adjoint {ad:.6e} vs finite difference {fd:.6e}"


def test_gradient_map_names_follow_the_oracle_keys():
    """``engine.adjoint_gradient_maps`` (the order of fw_adjoint_backward's output arrays) names
    the same maps, in the same order, as the FP64 adjoint's keys, for every engine."""
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    from fullwave25_gb300.engine import ADJOINT_MAPS, adjoint_gradient_maps

    assert adjoint_gradient_maps(load_case_inputs("2d_small")) == GRAD_KEYS == ADJOINT_MAPS
    assert adjoint_gradient_maps(load_case_inputs("2d_air_beta")) == GRAD_KEYS + ("beta2dt",)
    for name, nd in (("2d_aniso", 2), ("3d_aniso", 3)):
        assert adjoint_gradient_maps(load_case_inputs(name)) == aniso_grad_keys(nd)
    assert len(aniso_grad_keys(3)) == 32
