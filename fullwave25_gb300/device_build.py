"""Pre-processing on the GPU for the ``Solver`` path: from the physical description (grid,
medium, source, sensor) to the engine's inputs, built with torch on the device.

The reference does this on the host for every ``Solver.run()``: ``PMLBuilder`` pads every map
and ramps the relaxation parameters into the PML (fullwave/solver/pml_builder.py:270-276,
:321-704, :842-1254, :1256-1498), ``relaxation_parameters`` looks (alpha0, gamma) up in the
relaxation table (fullwave/solver/utils/relaxation_parameters.py:18-75), ``MediumRelaxationMaps``
sorts the mechanisms and forms the recursive-convolution coefficients (fullwave/medium.py:
121-209, :273-289), and ``InputFileWriter`` writes K, the tap tables and the coordinates
(fullwave/solver/input_file_writer.py:183-559, :716-862). Here the per-cell work runs on the
device in float64 with the same operations in the same order as this package's host builders
(``pml.PMLBuilder``, ``exponential.PMLBuilderExponentialAttenuation``, ``inputs.build_inputs``),
which restate the reference byte for byte; the float32 maps handed to the engine are equal to the
host builders' (checked element by element on the golden cases). What stays on the host is
O(boundary): the tap table (one entry per integer sound speed), and the source, sensor and air
coordinates, whose row-major order defines the rows of ``icmat`` and the trace columns.
"""

from __future__ import annotations

import time

import numpy as np

from . import coefficients
from .coords import map_to_coords
from .grid import Grid
from .medium import Medium, MediumRelaxationMaps, relaxation_param_keys
from .workloads3d import DeviceInputs, calc_a_and_b_t, extend_edge, pml_relaxation_maps_t


def _torch():
    import torch  # noqa: PLC0415

    return torch


def extended_grid(grid: Grid, shape, n_boundary: int) -> Grid:
    """The PML-extended grid, constructed as the PML builders construct it."""
    spacing = (grid.dx, grid.dy, grid.dz)
    domain = tuple((shape[k] + 2 * n_boundary) * spacing[k] for k in range(len(shape)))
    return Grid(domain_size=domain, f0=grid.f0, duration=grid.duration, c0=grid.c0,
                ppw=grid.ppw, cfl=grid.cfl)


def sort_mechanisms_t(params: dict) -> dict:
    """Per-cell order of the two mechanisms by time constant d/kappa + alpha (medium.py:121-209):
    a strictly smaller second time constant swaps the pair, ties keep the given order."""
    torch = _torch()
    out = dict(params)
    for op in ("x1", "x2"):
        t1 = params[f"d_{op}_nu1"] / params[f"kappa_{op}"] + params[f"alpha_{op}_nu1"]
        t2 = params[f"d_{op}_nu2"] / params[f"kappa_{op}"] + params[f"alpha_{op}_nu2"]
        swap = t2 < t1
        for var in ("d", "alpha"):
            a, b = params[f"{var}_{op}_nu1"], params[f"{var}_{op}_nu2"]
            out[f"{var}_{op}_nu1"] = torch.where(swap, b, a)
            out[f"{var}_{op}_nu2"] = torch.where(swap, a, b)
    return out


def relaxation_params_t(medium, device) -> dict:
    """Sorted relaxation parameter maps (float64, on the device) of a relaxation medium."""
    torch = _torch()
    t64 = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=device)  # noqa: E731
    if isinstance(medium, MediumRelaxationMaps):
        # already sorted by its constructor (the reference sorts there too)
        return {k: t64(v) for k, v in medium.relaxation_param_dict.items()}
    from .relaxation import default_table  # noqa: PLC0415
    from .workloads_batch import lookup_t  # noqa: PLC0415

    table = medium.relaxation_table or default_table()
    params = lookup_t(table, t64(medium.alpha_coeff), t64(medium.alpha_power))
    return sort_mechanisms_t({k: params[k] for k in relaxation_param_keys(2)})


def _fw_names(ndim: int, isotropic: bool) -> dict:
    """Engine map name -> coefficient key, as inputs.build_inputs names them."""
    from .inputs import DIV_AXIS_LETTER, GRAD_AXIS_LETTER  # noqa: PLC0415

    letters = ["u", "x"] if isotropic else (list(GRAD_AXIS_LETTER[:ndim])
                                            + list(DIV_AXIS_LETTER[:ndim]))
    names = {}
    for ax in letters:
        names[f"kappa{ax}"] = f"kappa_{ax}"
        for nu in (1, 2):
            names[f"apml{ax}{nu}"] = f"a_pml_{ax}{nu}"
            names[f"bpml{ax}{nu}"] = f"b_pml_{ax}{nu}"
    return names


def _coords(mask, n_boundary: int, ndim: int) -> np.ndarray:
    """Row-major coordinates of ``mask``'s cells on the extended grid (padding preserves order)."""
    return (map_to_coords(mask) + n_boundary).astype(np.int32).reshape(-1, ndim)


def device_inputs(grid: Grid, medium, source, sensor, *, n_pml: int, n_transition: int,
                  use_pml: bool = True, use_isotropic_relaxation: bool = True,
                  use_exponential_attenuation: bool = False, m_spatial_order: int = 8,
                  record_whole_domain: bool = False, sampling_modulus_time_whole_domain: int = 1,
                  device=None):
    """Engine inputs on the device; returns ``(DeviceInputs, n_sensors)``.

    ``medium``: a :class:`MediumRelaxationMaps`, or a :class:`Medium` (relaxation table lookup
    on the device, or the exponential-attenuation conversion when
    ``use_exponential_attenuation``). ``n_pml`` / ``n_transition``: PML and transition thickness
    in cells (the exponential engine pads by ``n_pml + m_spatial_order`` only, as its builder).
    """
    torch = _torch()
    t_start = time.perf_counter()
    device = device or torch.device("cuda", torch.cuda.current_device())
    t64 = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=device)  # noqa: E731
    shape = tuple(np.shape(medium.sound_speed))
    ndim = len(shape)
    if use_exponential_attenuation:
        nb = n_pml + m_spatial_order
    else:
        if not use_pml:
            n_pml = n_transition = 0
        elif n_pml == 0 or n_transition == 0:
            # the host builder ramps the second mechanism inside the transition layer and raises
            # without one (pml_builder.py:1281-1287 in the reference)
            raise ValueError("Transition layer is not defined. Set transit_within_transition_layer "
                             "to False or define n_transition_layer.")
        nb = n_pml + n_transition + m_spatial_order
    g = extended_grid(grid, shape, nb)
    c = extend_edge(t64(medium.sound_speed), nb)
    rho = extend_edge(t64(medium.density), nb)
    beta = extend_edge(t64(medium.beta), nb)
    maps = {"c": c.to(torch.float32), "rho": rho.to(torch.float32),
            "K": (c * c * rho).to(torch.float32), "beta": beta.to(torch.float32)}
    air = np.asarray(medium.air_map) if getattr(medium, "air_map", None) is not None else None
    if use_exponential_attenuation:
        if not isinstance(medium, Medium):
            raise TypeError("the exponential-attenuation engine needs a Medium (alpha_coeff)")
        maps["a_exp"] = _a_exp_t(extend_edge(t64(medium.alpha_coeff), nb), g, nb,
                                 use_pml).to(torch.float32)
        # the exponential builder pads the air map with edge values (pml_builder.py:1768-1778)
        air_ext = (np.pad(air, nb, mode="edge") if air is not None and air.any() else None)
        icczero = (map_to_coords(air_ext).astype(np.int32).reshape(-1, ndim) if air_ext is not None
                   else np.zeros((0, ndim), np.int32))
    else:
        params = {k: extend_edge(v, nb) for k, v in relaxation_params_t(medium, device).items()}
        if use_pml:
            fw2 = pml_relaxation_maps_t(params, n_pml=n_pml, n_transition=n_transition, dt=g.dt,
                                        c0=g.c0, dx=g.dx, ghost=m_spatial_order)
        else:
            fw2 = {"kappa_u": params["kappa_x1"], "kappa_x": params["kappa_x2"]}
            for nu in (1, 2):
                for ax, op in (("u", "x1"), ("x", "x2")):
                    fw2[f"a_pml_{ax}{nu}"], fw2[f"b_pml_{ax}{nu}"] = calc_a_and_b_t(
                        params[f"d_{op}_nu{nu}"], params[f"kappa_{op}"],
                        params[f"alpha_{op}_nu{nu}"], g.dt)
        del params
        if not use_isotropic_relaxation:
            # every derivative direction gets the ramps of every axis, so the per-direction sets
            # equal the isotropic gradient (u) and divergence (x) sets (pml_builder.py:60-89)
            from .inputs import DIV_AXIS_LETTER, GRAD_AXIS_LETTER  # noqa: PLC0415

            for a in range(1, ndim):
                for src, dst in (("u", GRAD_AXIS_LETTER[a]), ("x", DIV_AXIS_LETTER[a])):
                    fw2[f"kappa_{dst}"] = fw2[f"kappa_{src}"]
                    for nu in (1, 2):
                        fw2[f"a_pml_{dst}{nu}"] = fw2[f"a_pml_{src}{nu}"]
                        fw2[f"b_pml_{dst}{nu}"] = fw2[f"b_pml_{src}{nu}"]
        for name, key in _fw_names(ndim, use_isotropic_relaxation).items():
            maps[name] = fw2[key].to(torch.float32).contiguous()
        del fw2
        icczero = (_coords(air, nb, ndim) if air is not None else np.zeros((0, ndim), np.int32))
    cmin, cmax = float(c.min()), float(c.max())
    dmap = coefficients.d_map(np.array([cmin, cmax]), g.dt, g.dx, is_3d=ndim == 3)
    dcmap = (torch.round(c + 1e-9) - round(cmin + 1e-9)).to(torch.int32).contiguous()
    del c, rho, beta
    if record_whole_domain:
        ext_shape = tuple(n + 2 * nb for n in shape)
        outc = map_to_coords(np.ones(ext_shape, dtype=bool)).astype(np.int32)
        mod_t = int(sampling_modulus_time_whole_domain)
    else:
        outc = _coords(sensor.mask, nb, ndim)
        mod_t = int(sensor.sampling_modulus_time)
    i32 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32), device=device)  # noqa: E731
    icmat = torch.as_tensor(np.asarray(source.icmat, dtype=np.float32), device=device)
    spacing = (g.dx, g.dy, g.dz) if ndim == 3 else (g.dx, g.dy)
    if device.type == "cuda":
        torch.cuda.synchronize(device)
    d = DeviceInputs(shape=tuple(g.shape), nt=int(g.nt), spacing=spacing, dt=g.dt, c0=g.c0,
                     mod_t=mod_t, d=coefficients.d_matrix(g.cfl, is_3d=ndim == 3), dmap=dmap,
                     dcmap=dcmap, maps={k: v.contiguous() for k, v in maps.items()},
                     icc=i32(_coords(source.mask, nb, ndim)), icmat=icmat.contiguous(),
                     outc=i32(outc), icczero=i32(icczero),
                     build_s=time.perf_counter() - t_start)
    return d, int(outc.shape[0])


def _a_exp_t(alpha_ext, g: Grid, n_body: int, use_pml: bool):
    """``a_exp`` of the exponential engine (exponential.db_mhz_cm_to_a_exp and body_mask)."""
    torch = _torch()
    np_factor = -10 * np.log10(np.exp(-1))
    f0 = g.omega / (2.0 * np.pi * 1e6)
    texp = alpha_ext / 2.0 * f0 * g.c0 / (1e-2 * np_factor)
    a_exp = torch.exp(-g.dt * texp)
    if not use_pml:
        return a_exp
    r2 = 0
    for a, n in enumerate(a_exp.shape):
        idx = torch.arange(1, n + 1, device=a_exp.device).reshape(
            [-1 if b == a else 1 for b in range(a_exp.ndim)])
        r = torch.where(idx <= n_body, n_body - idx + 1,
                        torch.where(idx > n - n_body, idx - (n - n_body), 0))
        r2 = r2 + r ** 2
    mask = torch.sqrt(r2.to(torch.float64))
    if float(mask.max()) > 0:
        mask = mask / mask.max()
    return a_exp * (1 - mask)
