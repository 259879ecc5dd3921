"""GPU adjoint of the anisotropic relaxation engine (one relaxation map set per derivative axis;
2D and 3D, beta = 0) against the FP64 NumPy adjoint: all 2 + 10 ndim map gradients within 1e-3
relative L2, ghost cells zero; and the gradients of the raw per-direction maps through
``adjoint.map_gradients``."""

import numpy as np
import pytest

from fdtd_adjoint import aniso_grad_keys, misfit_and_gradient
from fdtd_oracle import GHOST, Oracle
from golden_io import load_case_inputs

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("name,nt,every", [("2d_aniso", 60, 25), ("3d_aniso", 36, 14)])
def test_anisotropic_map_gradients_match_fp64_adjoint(engine_lib, cuda, name, nt, every):
    torch = cuda
    from fullwave25_gb300.engine import Engine, adjoint_gradient_maps

    inp = _case(name, nt)
    observed = _observed(name, nt)
    _, G, _ = misfit_and_gradient(inp, observed)
    names = adjoint_gradient_maps(inp)
    assert names == aniso_grad_keys(len(inp.shape)) and len(names) == 2 + 10 * len(inp.shape)
    with Engine(inp) as eng:
        eng.adjoint_forward(every)
        res = torch.as_tensor(eng.read_traces() - observed.astype(np.float32),
                              device="cuda").contiguous()
        g = torch.zeros((len(names),) + tuple(inp.shape), dtype=torch.float64, device="cuda")
        eng.adjoint_backward(res.data_ptr(), g.data_ptr())
        torch.cuda.synchronize()
    g = g.cpu().numpy()
    body = tuple(slice(GHOST, n - GHOST) for n in inp.shape)
    for i, key in enumerate(names):
        ref = G[key]
        assert np.abs(ref).max() > 0, key
        err = np.linalg.norm(g[i][body] - ref) / np.linalg.norm(ref)
        assert err < 1e-3, f"{name} {key}: rel-L2 {err:.3e}"
        outside = g[i].copy()
        outside[body] = 0
        assert not outside.any()


def test_anisotropic_raw_map_gradients_through_the_python_layer(engine_lib, cuda):
    torch = cuda
    from fullwave25_gb300.adjoint import map_gradients
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads3d import DeviceInputs

    inp = _case("2d_aniso", 60)
    observed = _observed("2d_aniso", 60)
    _, G, _ = misfit_and_gradient(inp, observed)
    dev = torch.device("cuda", 0)
    t = lambda a: torch.as_tensor(np.ascontiguousarray(a), device=dev)  # noqa: E731
    dinp = DeviceInputs(shape=tuple(inp.shape), nt=inp.nt, spacing=inp.spacing, dt=inp.dt,
                        c0=inp.c0, mod_t=inp.mod_t, d=inp.d, dmap=inp.dmap, dcmap=t(inp.dcmap),
                        maps={k: t(v) for k, v in inp.maps.items()}, icc=t(inp.icc),
                        icmat=t(inp.icmat), outc=t(inp.outc), icczero=t(inp.icczero))
    with Engine(dinp, validate=False) as eng:
        J, traces, grads = map_gradients(eng, t(observed.astype(np.float32)), checkpoint_every=25)
    expect = {"rho", "K"} | {f"kappa{c}" for c in "uwxy"} | \
        {f"{ab}pml{c}{nu}" for ab in "ab" for c in "uwxy" for nu in (1, 2)}
    assert set(grads) == expect
    body = tuple(slice(GHOST, n - GHOST) for n in inp.shape)
    kw = inp.maps["kappaw"].astype(np.float64)[body]
    ref = G["inv_kw"] * (-1.0 / kw ** 2)
    got = grads["kappaw"].cpu().numpy()[body]
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-3
    got_a = grads["apmly2"].cpu().numpy()[body]
    assert np.linalg.norm(got_a - G["ay2"]) / np.linalg.norm(G["ay2"]) < 1e-3
