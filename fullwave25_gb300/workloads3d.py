"""Plain 3D forward workload built on the device (torch, float64 arithmetic, float32 result).

Geometry: 512^3 cells, dx = lambda/10 at f0 = 2 MHz (77 um), Courant 0.2, nt = 3000, PML 32 +
transition 32 cells per side -> 656^3 extended cells (282 M). Medium (seeded): fat
(c 1478, rho 950, alpha0 0.6, gamma 1.0), muscle (c 1547, rho 1050, alpha0 1.1, gamma 1.1), then
liver (c 1570, rho 1060, alpha0 0.5, gamma 1.2) along depth; each interface is displaced by a
Gaussian random field (sigma 1 mm, correlation length 3 mm); 0.5 % of the cells are scatterers
with +-2 % sound speed. Source: a 64 x 1 element linear array on depth row 0 (64 elements of
8 lateral cells, 32 elevation cells), all elements driven by the same 2 MHz pulse (plane wave).
Sensors: a 256 x 256 plane at depth row 4, recorded every step.

The PML extension and ramps are the same arithmetic as :mod:`fullwave25_gb300.pml` (which is
byte-checked against the reference's own pre-processing), written for torch tensors so that a
282 M-cell medium is built in seconds on the GPU; ``tests/test_workloads3d.py`` checks the two
implementations agree on a small grid.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from . import coefficients
from .grid import Grid
from .medium import relaxation_param_keys
from .pml import _transition
from .pulse import gaussian_modulated_sinusoidal_signal
from .relaxation import default_table

LAYERS = (  # name, c, rho, alpha0, gamma, top depth [m]
    ("fat", 1478.0, 950.0, 0.6, 1.0, 0.0),
    ("muscle", 1547.0, 1050.0, 1.1, 1.1, 8e-3),
    ("liver", 1570.0, 1060.0, 0.5, 1.2, 20e-3),
)


def _torch():
    import torch  # noqa: PLC0415

    return torch


def gaussian_random_field(shape, dx, sigma, corr_len, seed, device="cpu"):
    """2D Gaussian random field with Gaussian correlation ``corr_len`` and std ``sigma``."""
    torch = _torch()
    g = torch.Generator(device="cpu").manual_seed(seed)
    noise = torch.randn(shape, generator=g, dtype=torch.float64).to(device)
    ky = torch.fft.fftfreq(shape[0], d=dx, device=device, dtype=torch.float64)
    kz = torch.fft.fftfreq(shape[1], d=dx, device=device, dtype=torch.float64)
    k2 = ky[:, None] ** 2 + kz[None, :] ** 2
    filt = torch.exp(-(np.pi**2) * (corr_len**2) * k2 / 2)
    f = torch.fft.ifft2(torch.fft.fft2(noise) * filt).real
    return f / f.std() * sigma


def extend_edge(t, nb):
    """Edge-replicating padding by ``nb`` on every axis (as np.pad(mode='edge'))."""
    torch = _torch()
    idx = [torch.clamp(torch.arange(n + 2 * nb, device=t.device) - nb, 0, n - 1) for n in t.shape]
    out = t
    for a, ix in enumerate(idx):
        out = out.index_select(a, ix)
    return out


def extend_zero(t, nb):
    torch = _torch()
    return torch.nn.functional.pad(t, [nb] * (2 * t.ndim))


def ramp_axis_t(arr, target, axis, *, thickness, offset, kind, n_polynomial=2,
                ghost=coefficients.N_TAPS):
    """torch version of :func:`fullwave25_gb300.pml.ramp_axis` (same arithmetic and order)."""
    torch = _torch()
    out = arr.movedim(axis, 0)
    n = out.shape[0]
    tf = torch.as_tensor(_transition(kind, thickness, n_polynomial), dtype=arr.dtype,
                         device=arr.device)
    shape = (-1,) + (1,) * (out.ndim - 1)
    out[: ghost + offset + thickness] = target
    out[n - ghost - thickness - offset:] = target
    up_start, up_end = ghost + offset - 1, ghost + offset + thickness
    down_start, down_end = n - ghost - thickness - offset - 1, n - ghost - offset
    up_vals = out[up_end][None].clone()
    down_vals = out[down_start][None].clone()
    out[up_start:up_end] = up_vals - tf.flip(0).reshape(shape) * (up_vals - target)
    out[down_start:down_end] = down_vals - tf.reshape(shape) * (down_vals - target)
    return arr


def calc_a_and_b_t(d, kappa, alpha, dt):
    torch = _torch()
    b = torch.exp(-(d / kappa + alpha) * dt)
    a = d / (kappa * (d + kappa * alpha) + 1e-10) * (b - 1)
    return a, b


def pml_relaxation_maps_t(params: dict, *, n_pml, n_transition, dt, c0, dx,
                          ghost=coefficients.N_TAPS):
    """Ramped ``kappa*`` and ``a/b`` maps (isotropic) from extended float64 parameter maps.

    Same steps as :meth:`fullwave25_gb300.pml.PMLBuilder._apply_pml`.
    """
    ndim = params["kappa_x1"].ndim
    d_target = (-(2 + 1) * c0 * np.log(1e-30) / (2 * (dx * n_pml + dx * n_transition)))
    out = {}
    for ax, op in (("u", "x1"), ("x", "x2")):
        out[f"kappa_{ax}"] = params[f"kappa_{op}"]
        ramped = {}
        for nu in (1, 2):
            for var in ("alpha", "d"):
                arr = params[f"{var}_{op}_nu{nu}"].clone()
                for axis in range(ndim):
                    if nu == 1:
                        tgt = 0.0 if var == "alpha" else d_target
                        kind = "linear" if var == "alpha" else "polynomial"
                        arr = ramp_axis_t(arr, tgt, axis, thickness=n_pml + n_transition,
                                          offset=0, kind=kind, ghost=ghost)
                    else:
                        arr = ramp_axis_t(arr, 0.0, axis, thickness=n_transition, offset=n_pml,
                                          kind="cosine", ghost=ghost)
                ramped[(var, nu)] = arr
            out[f"a_pml_{ax}{nu}"], out[f"b_pml_{ax}{nu}"] = calc_a_and_b_t(
                ramped[("d", nu)], out[f"kappa_{ax}"], ramped[("alpha", nu)], dt)
    return out


@dataclass
class DeviceInputs:
    """Engine inputs held as CUDA tensors (maps float32, dcmap int32, coordinates int32)."""

    shape: tuple
    nt: int
    spacing: tuple
    dt: float
    c0: float
    mod_t: int
    d: np.ndarray
    dmap: np.ndarray
    dcmap: object
    maps: dict
    icc: object
    icmat: object
    outc: object
    icczero: object
    build_s: float = 0.0
    host_icmat: np.ndarray = field(default=None, repr=False)

    @property
    def ndim(self):
        return len(self.shape)

    @property
    def isotropic(self):
        return "kappay" not in self.maps

    @property
    def nt_ic(self):
        return int(self.icmat.shape[1])

    @property
    def n_out(self):
        return (self.nt + self.mod_t - 1) // self.mod_t

    def make_engine(self):
        from .engine import Engine  # noqa: PLC0415

        return Engine(self, validate=False)

    def run_e2e(self, engine, chunk, n_steps, stream_ptr, dev, world):
        """Per step: source columns of `chunk` time steps H2D from pinned memory, advance,
        sensor traces of those steps D2H into pinned memory (public C ABI throughout)."""
        torch = _torch()
        ncols = self.nt_ic
        # time-major pinned copy of the source signals: row n = samples of step n
        src_host = torch.empty((ncols, self.icmat.shape[0]), dtype=torch.float32,
                               pin_memory=True)
        src_host.copy_(self.icmat.t().cpu())
        out_host = torch.empty((chunk, self.outc.shape[0]), dtype=torch.float32, pin_memory=True)
        engine.reset(stream_ptr)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        h2d = d2h = 0
        for _ in range(n_steps):
            if engine.current_step + chunk > self.nt:
                engine.reset(stream_ptr)
            n0 = engine.current_step
            # the step's inputs: source samples for steps [n0, n0 + chunk)
            engine.set_source_columns(src_host[n0:n0 + chunk].numpy(), n0, stream_ptr)
            engine.advance(chunk, stream_ptr)
            r0 = n0 // self.mod_t
            nr = (n0 + chunk + self.mod_t - 1) // self.mod_t - r0
            engine.read_traces_to(out_host.numpy()[:nr], r0, stream_ptr)
            h2d = self.icmat.shape[0] * chunk * 4
            d2h = nr * self.outc.shape[0] * 4
        torch.cuda.synchronize(dev)
        el = time.perf_counter() - t0
        cells = int(np.prod(self.shape))
        return {"value": cells * chunk * n_steps * world / el / 1e9, "unit": "Gcell-updates/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "steps": n_steps,
                "api": "fw_set_source_columns(pinned host) + fw_advance + fw_read_traces(pinned host)"}


def layered_medium_3d(shape, dx, seed, device, n_boundary=0):
    """Sound speed, density and layer-id maps of the layered medium on the (extended) grid.

    ``n_boundary`` > 0 builds the maps directly on the PML-extended grid, replicating the
    original grid's edge cells outward exactly as edge padding would.
    """
    torch = _torch()
    nx, ny, nz = shape
    nb = n_boundary
    # interface depth fields over (y, z) of the original grid
    fields = [gaussian_random_field((ny, nz), dx, 1e-3, 3e-3, seed * 7 + k, device)
              for k in range(len(LAYERS) - 1)]
    cl = lambda n: torch.clamp(torch.arange(n + 2 * nb, device=device) - nb, 0, n - 1)  # noqa: E731
    ix, iy, iz = cl(nx), cl(ny), cl(nz)
    depth = (ix.to(torch.float64) * dx)[:, None, None]
    layer = torch.zeros((nx + 2 * nb, ny + 2 * nb, nz + 2 * nb), dtype=torch.int8, device=device)
    for k, lay in enumerate(LAYERS[1:], start=1):
        top = lay[5] + fields[k - 1][iy][:, iz]
        layer = torch.where(depth >= top[None], torch.tensor(k, dtype=torch.int8, device=device),
                            layer)
    c_tab = torch.tensor([l[1] for l in LAYERS], dtype=torch.float64, device=device)
    rho_tab = torch.tensor([l[2] for l in LAYERS], dtype=torch.float64, device=device)
    c = c_tab[layer.long()]
    rho = rho_tab[layer.long()]
    # scatterers: 0.5 % of the original grid's cells, +-2 % sound speed; a cell drawn twice takes
    # its last draw. The factor lives on the original grid and is edge-replicated like every map,
    # so the extended maps equal the padded original ones exactly.
    g = torch.Generator(device="cpu").manual_seed(seed * 7 + 100)
    n_scat = int(0.005 * nx * ny * nz)
    lin = torch.randint(0, nx * ny * nz, (n_scat,), generator=g).numpy()
    amp = ((torch.rand(n_scat, generator=g, dtype=torch.float64) * 2 - 1) * 0.02).numpy()
    _, last = np.unique(lin[::-1], return_index=True)
    keep = n_scat - 1 - last
    factor = torch.ones(nx * ny * nz, dtype=torch.float64, device=device)
    factor[torch.as_tensor(lin[keep], device=device)] = torch.as_tensor(1 + amp[keep], device=device)
    factor = factor.reshape(nx, ny, nz)
    if nb:
        factor = factor[ix][:, iy][:, :, iz]
    c = c * factor
    return c, rho, layer


def exp_attenuation_t(alpha0, grid, n_body: int):
    """``a_exp`` of the exponential-attenuation engine on the device: the amplitude fraction
    kept per update, ``exp(-dt * alpha0 / 2 * f0[MHz] * c0 / (1e-2 * 8.686))``
    (medium.py:1068-1090), scaled by ``1 - r`` inside the ``n_body``-cell padding, ``r`` the
    normalised distance into it (pml_builder.py:1800-1935; :func:`exponential.body_mask`)."""
    torch = _torch()
    np_factor = -10 * np.log10(np.exp(-1))
    texp = alpha0 / 2.0 * (grid.f0 / 1e6) * grid.c0 / (1e-2 * np_factor)
    a = torch.exp(-grid.dt * texp)
    r2 = torch.zeros((), dtype=torch.float64, device=alpha0.device)
    for ax, n in enumerate(a.shape):
        idx = torch.arange(1, n + 1, dtype=torch.float64, device=alpha0.device)
        r = torch.where(idx <= n_body, n_body - idx + 1,
                        torch.where(idx > n - n_body, idx - (n - n_body), torch.zeros_like(idx)))
        r2 = r2 + (r ** 2).reshape([-1 if b == ax else 1 for b in range(a.ndim)])
    mask = torch.sqrt(r2)
    if float(mask.max()) > 0:
        mask = mask / mask.max()
    return a * (1 - mask)


def plain_3d_device_inputs(seed: int = 0, shape=(512, 512, 512), nt: int = 3000,
                           f0: float = 2e6, ppw: int = 10, cfl: float = 0.2, n_pml: int = 32,
                           n_transition: int = 32, device=None, sensor_plane: int = 256,
                           element_height: int = 32, physics: str = "isotropic") -> DeviceInputs:
    """The plain 3D forward workload built on the device. ``physics``: "isotropic", "aniso"
    (one map set per derivative direction; the reference's anisotropic PML builder gives every
    direction the ramps of every axis, so the sets equal the isotropic ones,
    pml_builder.py:130-170), or "exp" (exponential attenuation from each layer's alpha0, on the
    same extended grid, ``a_exp`` ramped to zero over the boundary cells)."""
    torch = _torch()
    t_start = time.perf_counter()
    device = device or torch.device("cuda", torch.cuda.current_device())
    grid = Grid.from_cells(shape, f0=f0, nt=nt, ppw=ppw, cfl=cfl)
    nb = n_pml + n_transition + coefficients.N_TAPS
    ext = tuple(n + 2 * nb for n in shape)
    c, rho, layer = layered_medium_3d(shape, grid.dx, seed, device, n_boundary=nb)
    # relaxation parameters per layer from the lookup table, expanded per cell
    table = default_table()
    keys = relaxation_param_keys(2)
    per_layer = np.stack([np.array([table.lookup(np.array([[l[3]]]), np.array([[l[4]]]))[k][0, 0]
                                    for k in keys]) for l in LAYERS])
    plt = torch.as_tensor(per_layer, dtype=torch.float64, device=device)
    lid = layer.long()
    if physics == "exp":
        a0_tab = torch.tensor([l[3] for l in LAYERS], dtype=torch.float64, device=device)
        a_exp = exp_attenuation_t(a0_tab[lid], grid, nb).to(torch.float32)
    params = {k: plt[:, i][lid] for i, k in enumerate(keys)}
    # mechanism sort by time constant d/kappa + alpha (fullwave/medium.py:121-209)
    for op in ("x1", "x2"):
        tau1 = params[f"d_{op}_nu1"] / params[f"kappa_{op}"] + params[f"alpha_{op}_nu1"]
        tau2 = params[f"d_{op}_nu2"] / params[f"kappa_{op}"] + params[f"alpha_{op}_nu2"]
        swap = tau2 < tau1
        for var in ("d", "alpha"):
            a, b = params[f"{var}_{op}_nu1"], params[f"{var}_{op}_nu2"]
            params[f"{var}_{op}_nu1"], params[f"{var}_{op}_nu2"] = (torch.where(swap, b, a),
                                                                    torch.where(swap, a, b))
    del layer, lid
    fw2 = pml_relaxation_maps_t(params, n_pml=n_pml, n_transition=n_transition, dt=grid.dt,
                                c0=grid.c0, dx=grid.dx)
    del params
    names = {"kappax": "kappa_x", "kappau": "kappa_u"}
    for nu in (1, 2):
        for ax in ("u", "x"):
            names[f"apml{ax}{nu}"] = f"a_pml_{ax}{nu}"
            names[f"bpml{ax}{nu}"] = f"b_pml_{ax}{nu}"
    maps = {k: fw2[v].to(torch.float32).contiguous() for k, v in names.items()}
    del fw2
    if physics == "aniso":
        from .inputs import DIV_AXIS_LETTER, GRAD_AXIS_LETTER, axis_maps  # noqa: PLC0415

        for a in (1, 2):
            for src, dst in ((GRAD_AXIS_LETTER[0], GRAD_AXIS_LETTER[a]),
                             (DIV_AXIS_LETTER[0], DIV_AXIS_LETTER[a])):
                for ks, kd in zip(axis_maps(src), axis_maps(dst)):
                    maps[kd] = maps[ks].clone()
    elif physics == "exp":
        maps = {"a_exp": a_exp}
    elif physics != "isotropic":
        raise ValueError(f"unknown physics {physics!r}")
    maps["K"] = (c * c * rho).to(torch.float32)
    maps["rho"] = rho.to(torch.float32)
    maps["beta"] = torch.zeros(ext, dtype=torch.float32, device=device)
    # tap tables: dmap over the integer sound speeds present, dcmap per cell
    cmin, cmax = float(c.min()), float(c.max())
    span = int(coefficients.matlab_round(cmax) - coefficients.matlab_round(cmin))
    dmap = coefficients.d_map(np.array([cmin, cmax]), grid.dt, grid.dx, is_3d=True)
    assert dmap.shape[2] == span + 1
    dcmap = (torch.round(c + 1e-9) - round(cmin + 1e-9)).to(torch.int32)
    maps["c"] = c.to(torch.float32)
    del c, rho
    # source: 64 elements x 8 lateral cells, 32 elevation cells, on original depth row 0
    ny, nz = shape[1], shape[2]
    z0 = nz // 2 - element_height // 2
    yy, zz = np.meshgrid(np.arange(ny), np.arange(z0, z0 + element_height), indexing="ij")
    icc = np.stack([np.zeros(yy.size, dtype=np.int64), yy.ravel(), zz.ravel()], axis=1) + nb
    sig = gaussian_modulated_sinusoidal_signal(nt=nt, duration=grid.duration, ncycles=2,
                                               drop_off=2, f0=f0, p0=1e6).astype(np.float32)
    icmat = torch.as_tensor(sig, device=device)[None, :].expand(icc.shape[0], nt).contiguous()
    # sensors: central sensor_plane x sensor_plane at original depth row 4
    y0, zs0 = ny // 2 - sensor_plane // 2, nz // 2 - sensor_plane // 2
    sy, sz = np.meshgrid(np.arange(y0, y0 + sensor_plane), np.arange(zs0, zs0 + sensor_plane),
                         indexing="ij")
    outc = np.stack([np.full(sy.size, 4), sy.ravel(), sz.ravel()], axis=1) + nb
    to_i32 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32), device=device)  # noqa: E731
    if device.type == "cuda":
        torch.cuda.synchronize(device)
    return DeviceInputs(shape=ext, nt=nt, spacing=(grid.dx, grid.dy, grid.dz), dt=grid.dt,
                        c0=grid.c0, mod_t=1, d=coefficients.d_matrix(cfl, is_3d=True), dmap=dmap,
                        dcmap=dcmap.contiguous(), maps=maps, icc=to_i32(icc), icmat=icmat,
                        outc=to_i32(outc), icczero=to_i32(np.zeros((0, 3))),
                        build_s=time.perf_counter() - t_start)


def to_host_inputs(dinp: DeviceInputs):
    """Copy a :class:`DeviceInputs` to numpy :class:`EngineInputs` (for small grids)."""
    from .inputs import EngineInputs  # noqa: PLC0415

    return EngineInputs(shape=tuple(dinp.shape), nt=dinp.nt, spacing=dinp.spacing, dt=dinp.dt,
                        c0=dinp.c0, mod_t=dinp.mod_t, d=dinp.d, dmap=dinp.dmap,
                        dcmap=dinp.dcmap.cpu().numpy(),
                        maps={k: v.cpu().numpy() for k, v in dinp.maps.items()},
                        icc=dinp.icc.cpu().numpy(), icmat=dinp.icmat.cpu().numpy(),
                        outc=dinp.outc.cpu().numpy(), icczero=dinp.icczero.cpu().numpy())


def plain_3d_host_sample(edge: int = 48, nt: int = 3000, physics: str = "isotropic"):
    """A small block of the plain 3D medium (same layers, PML 8 + transition 8) as numpy inputs,
    used to time the FP64 oracle on the host."""
    torch = _torch()
    d = plain_3d_device_inputs(shape=(edge, edge, edge), nt=nt, n_pml=8, n_transition=8,
                               device=torch.device("cpu") if not torch.cuda.is_available()
                               else None, sensor_plane=16, element_height=8, physics=physics)
    return to_host_inputs(d)
