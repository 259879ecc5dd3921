"""GPU adjoint (FP32 wavefields; FP32 per-step contributions summed per checkpoint segment, FP64
time sums across segments) against the FP64 NumPy adjoint, against the all-FP64 accumulation
mode, and against central finite differences of the FP64 oracle.

Tolerances: engine-map gradients within 1e-3 relative L2 of the FP64 adjoint; physical-map
gradients (c, rho, alpha0) within 5e-3 of central differences (h = 1e-3 relative, tap sets
held fixed) at 16 random cells, relative to the larger of the two values plus 1e-6 of the
field's largest gradient.
"""

import numpy as np
import pytest

from fdtd_adjoint import GRAD_KEYS, misfit_and_gradient
from fdtd_oracle import GHOST, Oracle
from golden_io import load_case_inputs

pytestmark = pytest.mark.gpu


def _small(name, nt):
    inp = load_case_inputs(name)
    inp.nt = nt
    inp.icmat = np.ascontiguousarray(inp.icmat[:, :nt])
    return inp


@pytest.mark.parametrize("name,nt,every", [("2d_small", 90, 25), ("2d_nopml", 75, 75)])
def test_engine_map_gradients_match_fp64_adjoint(engine_lib, cuda, name, nt, every):
    torch = cuda
    from fullwave25_gb300.engine import ADJOINT_MAPS, Engine

    inp = _small(name, nt)
    obs_inp = _small(name, nt)
    obs_inp.maps = dict(obs_inp.maps)
    obs_inp.maps["K"] = (obs_inp.maps["K"] * np.float32(1.02)).astype(np.float32)
    observed = Oracle(obs_inp).run()
    J, G, traces64 = misfit_and_gradient(inp, observed)
    with Engine(inp) as eng:
        eng.adjoint_forward(every)
        traces = eng.read_traces()
        res = torch.as_tensor((traces - observed.astype(np.float32)), device="cuda").contiguous()
        g = torch.zeros((12,) + inp.shape, dtype=torch.float64, device="cuda")
        eng.adjoint_backward(res.data_ptr(), g.data_ptr())
        torch.cuda.synchronize()
    g = g.cpu().numpy()
    body = tuple(slice(GHOST, n - GHOST) for n in inp.shape)
    for i, key in enumerate(ADJOINT_MAPS):
        ref = G[key]
        got = g[i][body]
        err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert err < 1e-3, f"{name} {key}: rel-L2 {err:.3e}"
        outside = g[i].copy()
        outside[body] = 0
        assert not outside.any()


def test_segmented_accumulation_matches_fp64_steps(engine_lib, cuda):
    """Default accumulation (FP32 contributions, FP32 segment partials, FP64 totals) against
    every step formed and added in FP64 (FWGB_ADJ_F64_STEPS=1): within 1e-5 relative L2 per map,
    on a run with several segments."""
    import os

    torch = cuda
    from fullwave25_gb300.engine import Engine

    inp = _small("2d_small", 120)
    obs = _small("2d_small", 120)
    obs.maps = dict(obs.maps)
    obs.maps["rho"] = (obs.maps["rho"] * np.float32(0.97)).astype(np.float32)
    observed = Oracle(obs).run().astype(np.float32)
    out = {}
    for mode in ("segmented", "f64"):
        if mode == "f64":
            os.environ["FWGB_ADJ_F64_STEPS"] = "1"
        try:
            with Engine(inp) as eng:
                eng.adjoint_forward(30)
                res = torch.as_tensor(eng.read_traces() - observed, device="cuda").contiguous()
                g = torch.zeros((12,) + inp.shape, dtype=torch.float64, device="cuda")
                eng.adjoint_backward(res.data_ptr(), g.data_ptr())
                torch.cuda.synchronize()
                out[mode] = g.cpu().numpy()
        finally:
            os.environ.pop("FWGB_ADJ_F64_STEPS", None)
    for i in range(12):
        a, b = out["segmented"][i], out["f64"][i]
        assert np.abs(b).max() > 0
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err < 1e-5, f"map {i}: rel-L2 {err:.3e}"


@pytest.mark.parametrize("name", ["2d_small", "2d_air_beta_free"])
def test_reverse_step_forms_are_bitwise_equal(engine_lib, cuda, name):
    """The three forms of the reverse step give bitwise equal map gradients, also with air cells
    and sources: TMA-staged operands (default), two tiled launches with thread loads
    (FWGB_ADJ_TMA=0), and the five-launch form (FWGB_ADJ_FUSED=0)."""
    import os

    torch = cuda
    from fullwave25_gb300.engine import Engine

    base = "2d_small" if name == "2d_small" else "2d_air_beta"
    inp = _small(base, 100)
    if base == "2d_air_beta":   # the adjoint covers beta = 0; keep the air cells
        inp.maps = dict(inp.maps)
        inp.maps["beta"] = np.zeros_like(inp.maps["beta"])
    obs = _small(base, 100)
    obs.maps = dict(inp.maps)
    obs.maps["K"] = (obs.maps["K"] * np.float32(1.01)).astype(np.float32)
    observed = Oracle(obs).run().astype(np.float32)
    out = {}
    modes = {"tma": {}, "tiled": {"FWGB_ADJ_TMA": "0"}, "unfused": {"FWGB_ADJ_FUSED": "0"}}
    for mode, env in modes.items():
        os.environ.update(env)
        try:
            with Engine(inp) as eng:
                eng.adjoint_forward(25)
                res = torch.as_tensor(eng.read_traces() - observed, device="cuda").contiguous()
                g = torch.zeros((12,) + inp.shape, dtype=torch.float64, device="cuda")
                eng.adjoint_backward(res.data_ptr(), g.data_ptr())
                torch.cuda.synchronize()
                out[mode] = g.cpu().numpy()
        finally:
            for k in env:
                os.environ.pop(k, None)
    assert np.abs(out["unfused"]).max() > 0
    np.testing.assert_array_equal(out["tiled"], out["unfused"])
    np.testing.assert_array_equal(out["tma"], out["tiled"])


@pytest.mark.parametrize("shape,every,ghost_src", [((61, 83), 7, False), ((45, 120), 40, False),
                                                   ((45, 120), 40, True)])
def test_reverse_pass_variants_ragged(engine_lib, cuda, shape, every, ghost_src):
    """Reverse pass on grids whose body is not a whole number of 32 x 8 tiles (TMA boxes running
    past the array edge read zeros) and with checkpoint intervals that do not divide nt: TMA
    reverse step with out-of-place recomputation (default), tiled reverse step
    (FWGB_ADJ_TMA=0) and recomputation by state copies (FWGB_ADJ_OOP=0) give bitwise equal
    gradients. With a source in the ghost layer (pressure written there persists across steps)
    the engine recomputes by copies by itself, so the default matches too."""
    import os

    torch = cuda
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads import plain_2d_inputs

    def problem(scale):
        inp = plain_2d_inputs(shape=shape, nt=60, n_pml=6, n_transition=6)
        inp.maps = dict(inp.maps)
        inp.maps["rho"] = (inp.maps["rho"] * np.float32(scale)).astype(np.float32)
        if ghost_src:   # one more source row inside the ghost layer
            extra = np.stack([np.full(20, 3), np.arange(30, 50)], 1).astype(np.int32)
            inp.icc = np.concatenate([inp.icc, extra])
            inp.icmat = np.concatenate([inp.icmat, inp.icmat[:20]])
        return inp

    inp = problem(1.0)
    observed = Oracle(problem(1.03)).run().astype(np.float32)
    out = {}
    fields = {}
    modes = {"default": {}, "sequential": {"FWGB_ADJ_OVERLAP": "0"},
             "tiled": {"FWGB_ADJ_TMA": "0"}, "copies": {"FWGB_ADJ_OOP": "0"}}
    for mode, env in modes.items():
        os.environ.update(env)
        try:
            with Engine(inp) as eng:
                eng.adjoint_forward(every)
                res = torch.as_tensor(eng.read_traces() - observed, device="cuda").contiguous()
                g = torch.zeros((12,) + tuple(inp.shape), dtype=torch.float64, device="cuda")
                eng.adjoint_backward(res.data_ptr(), g.data_ptr())
                torch.cuda.synchronize()
                out[mode] = g.cpu().numpy()
                fields[mode] = eng.get_field(0)
        finally:
            for k in env:
                os.environ.pop(k, None)
    assert np.abs(out["copies"]).max() > 0
    for mode in ("default", "sequential", "tiled"):
        np.testing.assert_array_equal(out[mode], out["copies"], err_msg=mode)
        np.testing.assert_array_equal(fields[mode], fields["copies"], err_msg=mode)


def test_concurrent_gradients_with_different_tap_tables(engine_lib, cuda):
    """Gradient evaluations of handles whose tap tables differ in size (the reverse-step kernels'
    shared-memory needs differ) running at once, each on its own thread and stream: every result
    equals the same evaluation run alone."""
    import threading

    torch = cuda
    from fullwave25_gb300.workloads_batch import gradient_job

    jobs = [gradient_job(i, scale=0.12) for i in range(4)]
    sizes = {int(j.problem.build(*j.start).dmap.shape[-1]) for j in jobs}
    assert len(sizes) > 1
    alone = [j.run() for j in jobs]
    out = [None] * len(jobs)
    gate = threading.Barrier(len(jobs))

    def work(k):
        s = torch.cuda.Stream()
        gate.wait()
        for _ in range(2):
            out[k] = jobs[k].run(s)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(len(jobs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for k, (a, b) in enumerate(zip(alone, out)):
        assert b is not None, f"job {k} raised"
        assert a["J"] == b["J"] and a["J"] > 0
        for key, g in a["grads"].items():
            np.testing.assert_array_equal(b["grads"][key].cpu().numpy(), g.cpu().numpy(),
                                          err_msg=f"job {k} {key}")


@pytest.fixture(scope="module")
def problem(cuda):
    torch = cuda
    from fullwave25_gb300.adjoint import AdjointProblem
    from fullwave25_gb300.workloads import ellipse_medium_2d

    shape = (72, 64)
    c, rho, a0, gam = ellipse_medium_2d(shape, 1540 / 3e6 / 12, seed=11, n_ellipses=4)
    dev = torch.device("cuda")
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev)  # noqa: E731
    true = (t(c), t(rho), t(a0), t(gam))
    start = (t(np.full(shape, 1540.0)), t(np.full(shape, 1000.0)), t(np.full(shape, 0.5)), true[3])
    prob = AdjointProblem(shape, nt=420, n_pml=12, n_transition=12, c_ref=start[0],
                          device=dev, sensor_row=40)
    from fullwave25_gb300.engine import Engine

    with Engine(prob.build(*true), validate=False) as e:
        observed = torch.as_tensor(e.run(), device=dev)
    return prob, start, observed


def test_physical_gradients_match_finite_differences(engine_lib, cuda, problem):
    torch = cuda
    from fdtd_oracle_c import run_oracle_c
    from fullwave25_gb300.workloads3d import to_host_inputs

    prob, start, observed = problem
    c, rho, a0, gam = [x.clone().requires_grad_(i < 3) for i, x in enumerate(start)]
    J = prob.misfit(c, rho, a0, gam, observed, checkpoint_every=100)
    J.backward()
    grads = {"c": c.grad, "rho": rho.grad, "a0": a0.grad}
    obs = observed.cpu().numpy().astype(np.float64)

    def J64(cc, rr, aa):
        h = to_host_inputs(prob.build(cc, rr, aa, start[3]))
        tr = run_oracle_c(h)
        return 0.5 * float(np.sum((tr - obs) ** 2))

    rng = np.random.default_rng(3)
    nx, ny = prob.shape
    cells = [(int(rng.integers(0, nx)), int(rng.integers(0, ny))) for _ in range(16)]
    checked = 0
    for name, base in (("c", start[0]), ("rho", start[1]), ("a0", start[2])):
        gmax = float(grads[name].abs().max())
        for cell in (cells if name == "c" else cells[:4]):
            h = 1e-3 * abs(float(base[cell]))
            args = [start[0], start[1], start[2]]
            k = ("c", "rho", "a0").index(name)
            plus = [a.clone() for a in args]
            minus = [a.clone() for a in args]
            plus[k][cell] += h
            minus[k][cell] -= h
            fd = (J64(*plus) - J64(*minus)) / (2 * h)
            ad = float(grads[name][cell])
            # measured: c within 2e-5, alpha0 within 5e-6, rho within 1.8e-3 (relative); cells
            # whose gradient is ~1e-9 of the field's largest sit at the FP64 differences' noise
            assert abs(fd - ad) <= 5e-3 * max(abs(fd), abs(ad)) + 1e-6 * gmax, \
                f"d J / d {name} at {cell}: adjoint {ad:.6e}, finite difference {fd:.6e}"
            checked += 1
    assert checked == 24


def test_adjoint_rejects_sensor_groups(engine_lib, cuda):
    """The misfit is defined on individual sensor traces."""
    from fullwave25_gb300.engine import Engine, EngineError

    inp = _small("2d_small", 40)
    with Engine(inp) as e:
        n = inp.outc.shape[0]
        e.set_sensor_groups(np.arange(n) % 4, np.ones(n, dtype=np.float32), 4)
        with pytest.raises(EngineError, match="FW_ERR_UNSUPPORTED"):
            e.adjoint_forward(10)


def test_reverse_step_with_wide_tap_table(engine_lib, cuda):
    """2001 tap sets (sound speeds 1000-3000 m/s): the TMA reverse step copies a 96 KB tap table
    next to its tiles, the thread-load form reads the table from global memory; bitwise equal."""
    import os

    torch = cuda
    from fullwave25_gb300 import coefficients
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads import plain_2d_inputs

    def problem(scale):
        inp = plain_2d_inputs(shape=(50, 70), nt=60, n_pml=6, n_transition=6)
        c = np.random.default_rng(4).uniform(1000.0, 3000.0, size=inp.shape)
        c[0, 0], c[-1, -1] = 1000.0, 3000.0
        inp.maps = dict(inp.maps)
        inp.maps["c"] = c.astype(np.float32)
        inp.maps["K"] = (inp.maps["K"] * np.float32(scale)).astype(np.float32)
        inp.dmap = coefficients.d_map(c, inp.dt, inp.spacing[0], is_3d=False)
        inp.dcmap = coefficients.dc_map(c)
        return inp

    inp = problem(1.0)
    assert inp.dmap.shape[2] == 2001
    observed = Oracle(problem(1.02)).run().astype(np.float32)
    out = {}
    for mode, env in {"tma": {}, "tiled": {"FWGB_ADJ_TMA": "0"}}.items():
        os.environ.update(env)
        try:
            with Engine(inp) as eng:
                eng.adjoint_forward(20)
                res = torch.as_tensor(eng.read_traces() - observed, device="cuda").contiguous()
                g = torch.zeros((12,) + tuple(inp.shape), dtype=torch.float64, device="cuda")
                eng.adjoint_backward(res.data_ptr(), g.data_ptr())
                torch.cuda.synchronize()
                out[mode] = g.cpu().numpy()
        finally:
            for k in env:
                os.environ.pop(k, None)
    assert np.abs(out["tiled"]).max() > 0
    np.testing.assert_array_equal(out["tma"], out["tiled"])


def test_directional_derivative_at_benchmark_scale(engine_lib, cuda):
    """The benchmark's adjoint setup at 256^2 (432^2 extended, 1500 steps, 256 sensors, blurred
    start medium, checkpoints every 200 steps): the adjoint's derivative of J along a Gaussian
    bump in c (2 m/s, sigma 60 cells) equals the central difference of J computed by the FP64
    oracle within 1e-3 (measured 2e-5)."""
    torch = cuda
    from scipy.ndimage import gaussian_filter

    from fdtd_oracle_c import run_oracle_c
    from fullwave25_gb300.adjoint import AdjointProblem
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads import ellipse_medium_2d
    from fullwave25_gb300.workloads3d import to_host_inputs

    n, dev = 256, torch.device("cuda", 0)
    dx = 1540 / 3e6 / 12
    c, rho, a0, gam = ellipse_medium_2d((n, n), dx, seed=0)
    blur = lambda a: gaussian_filter(a, 2e-3 / dx, mode="nearest")  # noqa: E731
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev)  # noqa: E731
    start = (t(blur(c)), t(blur(rho)), t(blur(a0)), t(gam))
    prob = AdjointProblem((n, n), nt=1500, n_pml=40, n_transition=40, c_ref=start[0], device=dev,
                          sensor_row=5)
    with Engine(prob.build(t(c), t(rho), t(a0), t(gam)), validate=False) as e:
        observed = torch.as_tensor(e.run(), device=dev)
    cc = start[0].clone().requires_grad_(True)
    prob.misfit(cc, start[1], start[2], start[3], observed, checkpoint_every=200).backward()
    x = torch.arange(n, dtype=torch.float64, device=dev)[:, None] - (n - 1) / 2
    y = torch.arange(n, dtype=torch.float64, device=dev)[None, :] - (n - 1) / 2
    bump = 2.0 * torch.exp(-(x * x + y * y) / (2 * 60.0 ** 2))
    ad = float((cc.grad.double() * bump).sum())
    obs = observed.cpu().numpy().astype(np.float64)

    def J64(cv):
        tr = run_oracle_c(to_host_inputs(prob.build(cv, *start[1:])))
        return 0.5 * float(np.sum((tr - obs) ** 2))

    fd = (J64(start[0] + bump) - J64(start[0] - bump)) / 2.0
    assert abs(ad - fd) < 1e-3 * abs(fd), f"adjoint {ad:.6e}, central difference {fd:.6e}"
