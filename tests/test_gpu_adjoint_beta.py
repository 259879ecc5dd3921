"""GPU adjoint of the nonlinear engines (beta != 0; the pressure adjoint linearised around the
stored forward states) against the FP64 NumPy adjoint: every map gradient, 2 dt beta included
(the last gradient array), within 1e-3 relative L2; isotropic relaxation in 2D (with air cells
and a recording interval above 1) and 3D, the anisotropic and exponential engines in 2D."""

import numpy as np
import pytest

from fdtd_adjoint import misfit_and_gradient
from fdtd_oracle import GHOST, Oracle
from golden_io import load_case_inputs

pytestmark = pytest.mark.gpu
EXP_SLOT = {"rdt_rho": 0, "dt_k": 1, "a_exp": 4}


def _case(name, nt, beta=None):
    inp = load_case_inputs(name)
    inp.nt = nt
    inp.icmat = np.ascontiguousarray(inp.icmat[:, :nt])
    if beta is not None:
        inp.maps = dict(inp.maps)
        inp.maps["beta"] = np.full(inp.shape, beta, dtype=np.float32)
    return inp


@pytest.mark.parametrize("name,nt,every,beta", [("2d_air_beta", 60, 25, None),
                                                ("3d_small", 36, 14, 6.0),
                                                ("2d_aniso", 60, 25, 6.0),
                                                ("2d_exp", 60, 25, 8.0)])
def test_nonlinear_map_gradients_match_fp64_adjoint(engine_lib, cuda, name, nt, every, beta):
    torch = cuda
    from fullwave25_gb300.engine import Engine, adjoint_gradient_maps

    inp = _case(name, nt, beta)
    obs = _case(name, nt, beta)
    obs.maps = dict(obs.maps)
    obs.maps["K"] = (obs.maps["K"] * np.float32(1.02)).astype(np.float32)
    observed = Oracle(obs).run()
    _, G, _ = misfit_and_gradient(inp, observed)
    names = adjoint_gradient_maps(inp)
    assert names[-1] == "beta2dt"
    with Engine(inp) as eng:
        eng.adjoint_forward(every)
        res = torch.as_tensor(eng.read_traces() - observed.astype(np.float32),
                              device="cuda").contiguous()
        g = torch.zeros((len(names),) + tuple(inp.shape), dtype=torch.float64, device="cuda")
        eng.adjoint_backward(res.data_ptr(), g.data_ptr())
        torch.cuda.synchronize()
    g = g.cpu().numpy()
    body = tuple(slice(GHOST, n - GHOST) for n in inp.shape)
    exp = "a_exp" in inp.maps
    checks = ({**EXP_SLOT, "beta2dt": len(names) - 1} if exp
              else {k: i for i, k in enumerate(names)})
    for key, i in checks.items():
        ref = G[key]
        assert np.abs(ref).max() > 0, key
        err = np.linalg.norm(g[i][body] - ref) / np.linalg.norm(ref)
        assert err < 1e-3, f"{name} {key}: rel-L2 {err:.3e}"


def test_beta_set_between_adjoint_calls(engine_lib, cuda):
    """Setting a nonzero beta after fw_adjoint_forward adds a gradient map: the backward pass
    refuses the stale forward pass (FW_ERR_STATE) instead of writing past its buffers, and a new
    forward pass reallocates them for the extra map."""
    torch = cuda
    from fullwave25_gb300.engine import Engine, EngineError, adjoint_gradient_maps

    lin = _case("2d_small", 40)
    nonlin = _case("2d_small", 40, beta=6.0)
    observed = Oracle(nonlin).run().astype(np.float32)
    with Engine(lin) as eng:
        eng.adjoint_forward(15)
        eng.set_fields(nonlin)
        res = torch.zeros(observed.shape, dtype=torch.float32, device="cuda")
        g = torch.zeros((13,) + tuple(lin.shape), dtype=torch.float64, device="cuda")
        with pytest.raises(EngineError, match="FW_ERR_STATE"):
            eng.adjoint_backward(res.data_ptr(), g.data_ptr())
        names = adjoint_gradient_maps(nonlin)
        assert len(names) == 13
        eng.adjoint_forward(15)
        res = torch.as_tensor(eng.read_traces() - observed * 1.01, device="cuda").contiguous()
        eng.adjoint_backward(res.data_ptr(), g.data_ptr())
        torch.cuda.synchronize()
    assert np.isfinite(g.cpu().numpy()).all() and g[12].abs().max() > 0
