"""GPU adjoint of the 3D engine (isotropic relaxation, beta = 0; FP32 wavefields, FP32 per-step
contributions summed per checkpoint segment, FP64 time sums) against the FP64 NumPy adjoint,
against the all-FP64 accumulation mode, and against central differences of the FP64 C oracle.

Tolerances, as for the 2D adjoint: engine-map gradients within 1e-3 relative L2 of the FP64
adjoint; the default accumulation within 1e-5 of every step formed in FP64; the derivative of J
along a smooth bump in c within 1e-3 of the FP64 oracle's central difference.
"""

import os

import numpy as np
import pytest

from fdtd_adjoint import misfit_and_gradient
from fdtd_oracle import GHOST, Oracle
from golden_io import load_case_inputs

pytestmark = pytest.mark.gpu


def _case(nt):
    inp = load_case_inputs("3d_small")   # 44 x 42 x 40, sources and sensors in the body, modT 2
    inp.nt = nt
    inp.icmat = np.ascontiguousarray(inp.icmat[:, :nt])
    return inp


def _observed(nt, key, scale):
    obs = _case(nt)
    obs.maps = dict(obs.maps)
    obs.maps[key] = (obs.maps[key] * np.float32(scale)).astype(np.float32)
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


def test_3d_map_gradients_match_fp64_adjoint(engine_lib, cuda):
    """Every coefficient-map gradient of a 3D run (40 steps in checkpoint segments of 15, 15, 10)
    within 1e-3 relative L2 of the FP64 NumPy adjoint; ghost cells stay zero."""
    from fullwave25_gb300.engine import ADJOINT_MAPS

    inp = _case(40)
    observed = _observed(40, "K", 1.02)
    _, G, _ = misfit_and_gradient(inp, observed)
    g = _engine_gradients(cuda, inp, observed, every=15)
    body = tuple(slice(GHOST, n - GHOST) for n in inp.shape)
    for i, key in enumerate(ADJOINT_MAPS):
        ref = G[key]
        assert np.abs(ref).max() > 0
        err = np.linalg.norm(g[i][body] - ref) / np.linalg.norm(ref)
        assert err < 1e-3, f"3D {key}: rel-L2 {err:.3e}"
        outside = g[i].copy()
        outside[body] = 0
        assert not outside.any()


def test_3d_segmented_accumulation_matches_fp64_steps(engine_lib, cuda):
    """FP32 segment partials merged into FP64 sums against every step formed and added in FP64
    (FWGB_ADJ_F64_STEPS=1), within 1e-5 relative L2 per map."""
    inp = _case(48)
    observed = _observed(48, "rho", 0.97)
    a = _engine_gradients(cuda, inp, observed, every=16)
    b = _engine_gradients(cuda, inp, observed, every=16, env={"FWGB_ADJ_F64_STEPS": "1"})
    for i in range(12):
        assert np.abs(b[i]).max() > 0
        err = np.linalg.norm(a[i] - b[i]) / np.linalg.norm(b[i])
        assert err < 1e-5, f"map {i}: rel-L2 {err:.3e}"


def test_3d_directional_derivative_through_autograd(engine_lib, cuda):
    """A 3D medium (36 x 28 x 28, PML 10 + transition 10) with a Gaussian inclusion in c, rho and
    alpha0, sensed from a plane above it, against a homogeneous start: the derivative of J along a
    smooth bump in c from ``AdjointProblem.misfit(...).backward()`` equals the central difference
    of J from the FP64 C oracle within 1e-3."""
    torch = cuda
    from fdtd_oracle_c import run_oracle_c
    from fullwave25_gb300.adjoint import AdjointProblem
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads3d import to_host_inputs

    shape, dev = (36, 28, 28), torch.device("cuda", 0)
    g = [torch.arange(n, dtype=torch.float64, device=dev) for n in shape]
    x, y, z = torch.meshgrid(g[0] - 24, g[1] - 13.5, g[2] - 13.5, indexing="ij")
    blob = torch.exp(-(x * x + y * y + z * z) / (2 * 4.0 ** 2))
    ones = torch.ones(shape, dtype=torch.float64, device=dev)
    true = (1540.0 + 60.0 * blob, 1000.0 + 80.0 * blob, 0.5 + 0.4 * blob, 1.1 * ones)
    start = (1540.0 * ones, 1000.0 * ones, 0.5 * ones, 1.1 * ones)
    prob = AdjointProblem(shape, nt=300, n_pml=10, n_transition=10, c_ref=start[0], device=dev,
                          sensor_row=12, sensor_step=2)
    with Engine(prob.build(*true), validate=False) as e:
        observed = torch.as_tensor(e.run(), device=dev)
    cc = start[0].clone().requires_grad_(True)
    J = prob.misfit(cc, start[1], start[2], start[3], observed, checkpoint_every=64)
    J.backward()
    assert cc.grad.shape == shape and bool(torch.isfinite(cc.grad).all())
    bump = 2.0 * torch.exp(-((x + 4) ** 2 + y * y + z * z) / (2 * 6.0 ** 2))
    ad = float((cc.grad.double() * bump).sum())
    obs = observed.cpu().numpy().astype(np.float64)

    def J64(cv):
        tr = run_oracle_c(to_host_inputs(prob.build(cv, *start[1:])))
        return 0.5 * float(np.sum((tr - obs) ** 2))

    fd = (J64(start[0] + bump) - J64(start[0] - bump)) / 2.0
    assert abs(fd) > 0
    assert abs(ad - fd) < 1e-3 * abs(fd), f"adjoint {ad:.6e}, central difference {fd:.6e}"
