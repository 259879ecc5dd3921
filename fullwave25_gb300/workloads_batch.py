"""Batched 2D workload: many independent simulations of uneven sizes (built on the device).

Instance ``i`` (seed = i): grid depth x lateral drawn from {512, 768, 1024, 1536, 2048} x
{512, 1024, 1536} cells; f0 uniform in [3, 5] MHz, dx = lambda/12, Courant 0.2, PML 40 +
transition 40 cells; nt scaled linearly with depth from 3000 (512 cells) to 8000 (2048 cells);
medium as the plain 2D workload (background tissue plus eight seeded ellipses); transmit: a
128-element linear array on depth row 0 spanning the lateral extent, either a plane wave steered
by an angle in [-15, 15] degrees or a focused beam at 20-40 mm depth; receive: every lateral cell
of depth row 1, every step.
"""

from __future__ import annotations

import numpy as np

from . import coefficients
from .grid import Grid
from .medium import relaxation_param_keys
from .pulse import gaussian_modulated_sinusoidal_signal
from .relaxation import default_table
from .workloads3d import DeviceInputs, extend_edge, pml_relaxation_maps_t

DEPTHS = (512, 768, 1024, 1536, 2048)
WIDTHS = (512, 1024, 1536)
N_ELEMENTS = 128


def _torch():
    import torch  # noqa: PLC0415

    return torch


def instance_spec(i: int) -> dict:
    rng = np.random.default_rng(i)
    nx = int(rng.choice(DEPTHS))
    ny = int(rng.choice(WIDTHS))
    f0 = float(rng.uniform(3e6, 5e6))
    nt = int(round(3000 + (nx - 512) / (2048 - 512) * 5000))
    focused = bool(rng.integers(0, 2))
    angle = float(rng.uniform(-15, 15))
    focus = float(rng.uniform(20e-3, 40e-3))
    return {"nx": nx, "ny": ny, "f0": f0, "nt": nt, "focused": focused, "angle_deg": angle,
            "focus_m": focus, "seed": i}


def lookup_t(table, a0, gam):
    """Relaxation-table lookup on the device, same bins as RelaxationTable.lookup."""
    torch = _torch()
    al = torch.as_tensor(table.alpha_list.round(10), device=a0.device)
    pl = torch.as_tensor(table.power_list.round(10), device=a0.device)
    a = torch.clamp(a0, float(table.alpha_list.min()), float(table.alpha_list.max()))
    g = torch.clamp(gam, float(table.power_list.min()), float(table.power_list.max().round(4)))
    ia = torch.clamp(torch.searchsorted(al, a.contiguous()), 0, len(al) - 1)
    ig = torch.clamp(torch.searchsorted(pl, g.contiguous()), 0, len(pl) - 1)
    tab = torch.as_tensor(table.table, device=a0.device)
    out = tab[ia, ig]
    return {k: out[..., n] for n, k in enumerate(relaxation_param_keys(2))}


def ellipse_medium_2d_t(shape, dx, seed, device, n_ellipses=8):
    """Device version of :func:`fullwave25_gb300.workloads.ellipse_medium_2d` (same draws)."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    nx, ny = shape
    c = torch.full(shape, 1540.0, dtype=torch.float64, device=device)
    rho = torch.full(shape, 1000.0, dtype=torch.float64, device=device)
    a0 = torch.full(shape, 0.5, dtype=torch.float64, device=device)
    gam = torch.full(shape, 1.1, dtype=torch.float64, device=device)
    x = (torch.arange(nx, device=device, dtype=torch.float64) * dx)[:, None]
    y = (torch.arange(ny, device=device, dtype=torch.float64) * dx)[None, :]
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


def transmit_delays(spec, dx, c0=1540.0):
    """Per-element firing delays [s] (non-negative) of the 128-element array."""
    ny = spec["ny"]
    y = (np.arange(N_ELEMENTS) + 0.5) * (ny / N_ELEMENTS) * dx
    yc = ny * dx / 2
    if spec["focused"]:
        dist = np.sqrt((y - yc) ** 2 + spec["focus_m"] ** 2)
        d = (dist.max() - dist) / c0
    else:
        d = (y - y[0]) * np.sin(np.deg2rad(spec["angle_deg"])) / c0
        d = d - d.min()
    return d


def batch_instance(i: int, device=None, n_pml: int = 40, n_transition: int = 40,
                   scale: float = 1.0) -> DeviceInputs:
    """Device inputs of batch instance ``i`` (``scale`` < 1 shrinks the grid for tests)."""
    torch = _torch()
    device = device or torch.device("cuda", torch.cuda.current_device())
    spec = instance_spec(i)
    nx = max(32, int(spec["nx"] * scale))
    ny = max(N_ELEMENTS, int(spec["ny"] * scale) // N_ELEMENTS * N_ELEMENTS)
    nt = max(50, int(spec["nt"] * scale))
    spec = {**spec, "nx": nx, "ny": ny, "nt": nt}
    grid = Grid.from_cells((nx, ny), f0=spec["f0"], nt=nt, ppw=12, cfl=0.2)
    nb = n_pml + n_transition + coefficients.N_TAPS
    c, rho, a0, gam = ellipse_medium_2d_t((nx, ny), grid.dx, spec["seed"], device)
    params = lookup_t(default_table(), a0, gam)
    for op in ("x1", "x2"):  # mechanism sort by time constant (fullwave/medium.py:121-209)
        t1 = params[f"d_{op}_nu1"] / params[f"kappa_{op}"] + params[f"alpha_{op}_nu1"]
        t2 = params[f"d_{op}_nu2"] / params[f"kappa_{op}"] + params[f"alpha_{op}_nu2"]
        sw = t2 < t1
        for var in ("d", "alpha"):
            a, b = params[f"{var}_{op}_nu1"], params[f"{var}_{op}_nu2"]
            params[f"{var}_{op}_nu1"], params[f"{var}_{op}_nu2"] = (torch.where(sw, b, a),
                                                                    torch.where(sw, a, b))
    params = {k: extend_edge(v, nb) for k, v in params.items()}
    c, rho = extend_edge(c, nb), extend_edge(rho, nb)
    fw2 = pml_relaxation_maps_t(params, n_pml=n_pml, n_transition=n_transition, dt=grid.dt,
                                c0=grid.c0, dx=grid.dx)
    names = {"kappax": "kappa_x", "kappau": "kappa_u"}
    for nu in (1, 2):
        for ax in ("u", "x"):
            names[f"apml{ax}{nu}"] = f"a_pml_{ax}{nu}"
            names[f"bpml{ax}{nu}"] = f"b_pml_{ax}{nu}"
    maps = {k: fw2[v].to(torch.float32).contiguous() for k, v in names.items()}
    maps["K"] = (c * c * rho).to(torch.float32)
    maps["rho"] = rho.to(torch.float32)
    maps["beta"] = torch.zeros_like(maps["rho"])
    maps["c"] = c.to(torch.float32)
    cmin, cmax = float(c.min()), float(c.max())
    dmap = coefficients.d_map(np.array([cmin, cmax]), grid.dt, grid.dx, is_3d=False)
    dcmap = (torch.round(c + 1e-9) - round(cmin + 1e-9)).to(torch.int32).contiguous()
    # transmit: element e covers lateral cells [e*w, (e+1)*w) of depth row 0; the element
    # signals (all delays at once) go to the device, which repeats them over the element's cells
    w = ny // N_ELEMENTS
    delays = transmit_delays(spec, grid.dx)
    sig = gaussian_modulated_sinusoidal_signal(
        nt=nt, duration=grid.duration, ncycles=2, drop_off=2, f0=spec["f0"], p0=1e6,
        delay_sec=delays[:, None]).astype(np.float32)
    cols = np.arange(N_ELEMENTS * w)
    icc = np.stack([np.zeros_like(cols), cols], axis=1) + nb
    icmat = torch.as_tensor(sig, device=device).repeat_interleave(w, dim=0)
    outc = np.stack([np.ones(ny, dtype=np.int64), np.arange(ny)], axis=1) + nb
    i32 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32), device=device)  # noqa: E731
    d = DeviceInputs(shape=(nx + 2 * nb, ny + 2 * nb), nt=nt, spacing=(grid.dx, grid.dy),
                     dt=grid.dt, c0=grid.c0, mod_t=1, d=coefficients.d_matrix(0.2, is_3d=False),
                     dmap=dmap, dcmap=dcmap, maps=maps, icc=i32(icc), icmat=icmat.contiguous(),
                     outc=i32(outc), icczero=i32(np.zeros((0, 2))))
    d.spec = spec
    return d


def batch_problem_host(i: int, n_pml: int = 40, n_transition: int = 40, scale: float = 1.0):
    """Instance ``i`` through the host-side API (the reference's call sequence): Grid, a NumPy
    medium with the same seeded draws, relaxation-table lookup, Source/Sensor masks; returns
    (grid, medium, source, sensor, (n_pml, n_transition)) for :class:`PMLBuilder` /
    :class:`fullwave25_gb300.Solver`. Same physics as :func:`batch_instance`."""
    from .medium import MediumRelaxationMaps  # noqa: PLC0415
    from .source import Sensor, Source  # noqa: PLC0415
    from .workloads import ellipse_medium_2d  # noqa: PLC0415

    spec = instance_spec(i)
    nx = max(32, int(spec["nx"] * scale))
    ny = max(N_ELEMENTS, int(spec["ny"] * scale) // N_ELEMENTS * N_ELEMENTS)
    nt = max(50, int(spec["nt"] * scale))
    spec = {**spec, "nx": nx, "ny": ny, "nt": nt}
    grid = Grid.from_cells((nx, ny), f0=spec["f0"], nt=nt, ppw=12, cfl=0.2)
    c, rho, a0, gam = ellipse_medium_2d((nx, ny), grid.dx, seed=spec["seed"])
    medium = MediumRelaxationMaps(grid, c, rho, np.zeros((nx, ny)),
                                  default_table().lookup(a0, gam))
    w = ny // N_ELEMENTS
    sig = np.stack([gaussian_modulated_sinusoidal_signal(
        nt=nt, duration=grid.duration, ncycles=2, drop_off=2, f0=spec["f0"], p0=1e6,
        delay_sec=float(d)) for d in transmit_delays(spec, grid.dx)])
    mask = np.zeros((nx, ny), dtype=bool)
    mask[0, :N_ELEMENTS * w] = True
    source = Source(np.repeat(sig, w, axis=0), mask)
    smask = np.zeros((nx, ny), dtype=bool)
    smask[1, :] = True
    sensor = Sensor(smask, sampling_modulus_time=1)
    return grid, medium, source, sensor, (n_pml, n_transition)


def batch_inputs_host(i: int, **kw):
    """Host :class:`EngineInputs` of instance ``i`` built by the NumPy pre-processing path."""
    from .inputs import build_inputs  # noqa: PLC0415
    from .pml import PMLBuilder  # noqa: PLC0415

    grid, medium, source, sensor, (n_pml, n_tr) = batch_problem_host(i, **kw)
    b = PMLBuilder(grid, medium, source, sensor, n_pml_layer=n_pml, n_transition_layer=n_tr)
    return build_inputs(b.extended_grid, b.run(), b.extended_source, b.extended_sensor)


GRADIENT_SIZES = (512, 768, 1024)


def gradient_job(i: int, scale: float = 1.0, device=None, checkpoint_every: int = 200):
    """Gradient request ``i`` of the serving mix (seed = i): a square grid drawn from
    {512, 768, 1024}^2 (times ``scale``), nt = 6000 at 1024 scaled with the grid, f0 = 3 MHz,
    sensors every other cell of depth row 5; the starting medium is the seeded true medium
    Gaussian-blurred with sigma = 2 mm, and the observed traces are the true medium's forward
    solve (computed here, as the request's input data)."""
    from scipy.ndimage import gaussian_filter  # noqa: PLC0415

    from .adjoint import AdjointProblem  # noqa: PLC0415
    from .engine import Engine  # noqa: PLC0415
    from .server import GradientJob  # noqa: PLC0415
    from .workloads import ellipse_medium_2d  # noqa: PLC0415

    torch = _torch()
    device = device or torch.device("cuda", torch.cuda.current_device())
    rng = np.random.default_rng(10_000 + i)
    n = max(64, int(int(rng.choice(GRADIENT_SIZES)) * scale))
    nt = max(100, int(round(6000 * n / 1024)))
    dx = 1540 / 3e6 / 12
    c, rho, a0, gam = ellipse_medium_2d((n, n), dx, seed=10_000 + i)
    sig = 2e-3 / dx
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=device)  # noqa: E731
    blur = lambda a: t(gaussian_filter(a, sig, mode="nearest"))  # noqa: E731
    start = (blur(c), blur(rho), blur(a0), t(gam))
    prob = AdjointProblem((n, n), nt=nt, n_pml=40, n_transition=40, c_ref=start[0],
                          device=device, sensor_step=2, sensor_row=5)
    with Engine(prob.build(t(c), t(rho), t(a0), t(gam)), validate=False) as e:
        observed = torch.as_tensor(e.run(), device=device)
    return GradientJob(problem=prob, start=start, observed=observed,
                       checkpoint_every=min(checkpoint_every, nt))
