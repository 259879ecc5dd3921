"""GPU adjoint of the exponential-attenuation engine (2D and 3D, beta = 0) against the FP64 NumPy
adjoint: gradients with respect to dt/rho, dt*K and a_exp (returned in the au1 slot, the map slot
the engine keeps a_exp in; every other slot stays zero) within 1e-3 relative L2, and the default
accumulation (FP32 segment partials) within 1e-5 of every step formed in FP64."""

import os

import numpy as np
import pytest

from fdtd_adjoint import misfit_and_gradient
from fdtd_oracle import GHOST, Oracle
from golden_io import load_case_inputs

pytestmark = pytest.mark.gpu
SLOT = {"rdt_rho": 0, "dt_k": 1, "a_exp": 4}


def _case(name, nt):
    inp = load_case_inputs(name)
    inp.nt = nt
    inp.icmat = np.ascontiguousarray(inp.icmat[:, :nt])
    return inp


def _observed(name, nt):
    obs = _case(name, nt)
    obs.maps = dict(obs.maps)
    obs.maps["K"] = (obs.maps["K"] * np.float32(1.02)).astype(np.float32)
    return Oracle(obs).run()


def _engine_gradients(torch, inp, observed, every, env=None):
    from fullwave25_gb300.engine import Engine

    env = env or {}
    os.environ.update(env)
    try:
        with Engine(inp) as eng:
            eng.adjoint_forward(every)
            res = torch.as_tensor(eng.read_traces() - observed.astype(np.float32),
                                  device="cuda").contiguous()
            g = torch.zeros((12,) + tuple(inp.shape), dtype=torch.float64, device="cuda")
            eng.adjoint_backward(res.data_ptr(), g.data_ptr())
            torch.cuda.synchronize()
    finally:
        for k in env:
            os.environ.pop(k, None)
    return g.cpu().numpy()


@pytest.mark.parametrize("name,nt,every", [("2d_exp", 60, 25), ("3d_exp", 40, 15)])
def test_exponential_map_gradients_match_fp64_adjoint(engine_lib, cuda, name, nt, every):
    inp = _case(name, nt)
    observed = _observed(name, nt)
    _, G, _ = misfit_and_gradient(inp, observed)
    g = _engine_gradients(cuda, inp, observed, every)
    body = tuple(slice(GHOST, n - GHOST) for n in inp.shape)
    for key, i in SLOT.items():
        ref = G[key]
        assert np.abs(ref).max() > 0
        err = np.linalg.norm(g[i][body] - ref) / np.linalg.norm(ref)
        assert err < 1e-3, f"{name} {key}: rel-L2 {err:.3e}"
        outside = g[i].copy()
        outside[body] = 0
        assert not outside.any()
    for i in set(range(12)) - set(SLOT.values()):
        assert not g[i].any(), f"slot {i} should stay zero"


def test_exponential_segmented_accumulation_matches_fp64_steps(engine_lib, cuda):
    inp = _case("2d_exp", 80)
    observed = _observed("2d_exp", 80)
    a = _engine_gradients(cuda, inp, observed, every=20)
    b = _engine_gradients(cuda, inp, observed, every=20, env={"FWGB_ADJ_F64_STEPS": "1"})
    for i in SLOT.values():
        assert np.abs(b[i]).max() > 0
        err = np.linalg.norm(a[i] - b[i]) / np.linalg.norm(b[i])
        assert err < 1e-5, f"slot {i}: rel-L2 {err:.3e}"


def test_exponential_map_gradients_through_the_python_layer(engine_lib, cuda):
    """``adjoint.map_gradients`` on an exponential engine returns the gradients of the raw maps
    rho, K and a_exp (chained from dt/rho, dt*K, a_exp)."""
    torch = cuda
    from fullwave25_gb300.adjoint import map_gradients
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads3d import DeviceInputs

    inp = _case("2d_exp", 60)
    observed = _observed("2d_exp", 60)
    _, G, _ = misfit_and_gradient(inp, observed)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)  # noqa: E731
    dinp = DeviceInputs(shape=tuple(inp.shape), nt=inp.nt, spacing=inp.spacing, dt=inp.dt,
                        c0=inp.c0, mod_t=inp.mod_t, d=inp.d, dmap=inp.dmap, dcmap=t(inp.dcmap),
                        maps={k: t(v) for k, v in inp.maps.items()}, icc=t(inp.icc),
                        icmat=t(inp.icmat), outc=t(inp.outc), icczero=t(inp.icczero))
    with Engine(dinp, validate=False) as eng:
        J, traces, grads = map_gradients(eng, t(observed.astype(np.float32)), checkpoint_every=25)
    assert set(grads) == {"rho", "K", "a_exp"}
    body = tuple(slice(GHOST, n - GHOST) for n in inp.shape)
    ref = G["a_exp"]
    got = grads["a_exp"].cpu().numpy()[body]
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-3
    dt = float(np.float32(inp.dt))
    ref_k = G["dt_k"] * dt
    got_k = grads["K"].cpu().numpy()[body]
    assert np.linalg.norm(got_k - ref_k) / np.linalg.norm(ref_k) < 1e-3
