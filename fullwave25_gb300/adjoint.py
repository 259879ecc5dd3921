"""Gradients of the sensor-trace misfit with respect to sound speed, density and alpha0 (2D, 3D).

Layers:
1. :func:`map_gradients` runs the engine's checkpointed forward pass and its discrete adjoint
   (``fw_adjoint_forward`` / ``fw_adjoint_backward``): the misfit ``J = 1/2 sum (traces -
   observed)^2`` reduced in FP64 on the GPU, and the FP64 time-summed gradient of ``J`` with
   respect to every coefficient map the time loop multiplies by, chained to the raw input maps
   (rho, K, kappau, kappax, apml*, bpml*).
2. :class:`FdtdMisfit` is a ``torch.autograd.Function`` over those raw maps.
3. :class:`AdjointProblem` builds the raw maps from physical ``c``, ``rho``, ``alpha0`` (and a fixed
   ``gamma``) on the original grid with differentiable torch operations (PML padding and ramps
   as in :mod:`fullwave25_gb300.pml`), so ``J.backward()`` yields dJ/dc, dJ/drho, dJ/dalpha0.

The per-cell tap set (``dcmap``, the integer sound speed) is held fixed at the starting medium:
it is piecewise constant in c and contributes no gradient almost everywhere. Relaxation
strengths are linear in alpha0 at fixed gamma (``d_nu = alpha0 * d_nu(1, gamma)``, exact for the
stand-in lookup table), so alpha0 has a gradient; the relaxation rates depend on gamma only.
"""

from __future__ import annotations

import dataclasses

import numpy as np

from . import coefficients
from .engine import Engine, adjoint_gradient_maps
from .grid import Grid
from .medium import relaxation_param_keys
from .relaxation import default_table
from .workloads3d import DeviceInputs, extend_edge, pml_relaxation_maps_t

RAW_MAPS = ("rho", "K", "kappau", "kappax", "apmlu1", "bpmlu1", "apmlu2", "bpmlu2",
            "apmlx1", "bpmlx1", "apmlx2", "bpmlx2")


def _torch():
    import torch  # noqa: PLC0415

    return torch


def map_gradients(engine: Engine, observed, checkpoint_every: int = 200, stream=None):
    """Misfit and raw-map gradients for ``engine`` (its current fields) against ``observed``.

    ``observed``: CUDA float32 tensor ``[n_out, ncoordsout]``. ``stream``: a torch CUDA stream
    (None: the current one); all work is ordered on it and only it is synchronised, so gradient
    evaluations on other streams overlap. Returns ``(J, traces, grads)`` with ``grads[name]`` a
    float64 CUDA tensor of the grid shape for every name in ``RAW_MAPS`` (and ``beta`` when the
    beta map is not zero everywhere); for the
    exponential-attenuation engine (inputs with an ``a_exp`` map) for ``rho``, ``K`` and
    ``a_exp``; for the anisotropic engine for ``rho``, ``K`` and every per-direction map
    (``kappa{u,w,v,x,y,z}``, ``apml*``, ``bpml*``).
    """
    torch = _torch()
    inp = engine.inputs
    dev = observed.device
    ts = stream if stream is not None else torch.cuda.current_stream(dev)
    raw = ts.cuda_stream
    with torch.cuda.stream(ts):
        engine.adjoint_forward(checkpoint_every, raw)
        traces = torch.empty_like(observed)
        engine.read_traces_into(0, inp.n_out, traces.data_ptr(), raw)
        residual = (traces - observed).contiguous()
        J = 0.5 * float(torch.sum(residual.double() ** 2))
        names = adjoint_gradient_maps(inp)
        g = torch.zeros((len(names),) + tuple(inp.shape), dtype=torch.float64, device=dev)
        engine.adjoint_backward(residual.data_ptr(), g.data_ptr(), raw)
        gm = dict(zip(names, g))
        dt = float(np.float32(inp.dt))
        extra = {"beta": gm["beta2dt"] * (2.0 * dt)} if "beta2dt" in gm else {}

        def dmap(k):   # an input map as a float64 tensor on the device (numpy or torch inputs)
            return torch.as_tensor(inp.maps[k], device=dev).double()

        if "kappay" in inp.maps:   # anisotropic engine: per-direction map sets
            rho = dmap("rho")
            grads = {"rho": gm["rdt_rho"] * (-dt / rho ** 2), "K": gm["dt_k"] * dt}
            for n in names[2:]:
                if n.startswith("inv_k"):
                    kap = dmap(f"kappa{n[5]}")
                    grads[f"kappa{n[5]}"] = gm[n] * (-1.0 / kap ** 2)
                elif n != "beta2dt":
                    grads[f"{n[0]}pml{n[1:]}"] = gm[n]
            grads.update(extra)
            ts.synchronize()
            return J, traces, grads
        if "a_exp" in inp.maps:   # exponential engine: a_exp sits in the au1 slot
            rho = dmap("rho")
            grads = {"rho": gm["rdt_rho"] * (-dt / rho ** 2), "K": gm["dt_k"] * dt,
                     "a_exp": gm["au1"], **extra}
            ts.synchronize()
            return J, traces, grads
        m = {k: dmap(k) for k in ("rho", "K", "kappau", "kappax")}
        grads = {
            "rho": gm["rdt_rho"] * (-dt / m["rho"] ** 2),
            "K": gm["dt_k"] * dt,
            "kappau": gm["inv_ku"] * (-1.0 / m["kappau"] ** 2),
            "kappax": gm["inv_kx"] * (-1.0 / m["kappax"] ** 2),
        }
        for nu in (1, 2):
            for ax in ("u", "x"):
                grads[f"apml{ax}{nu}"] = gm[f"a{ax}{nu}"]
                grads[f"bpml{ax}{nu}"] = gm[f"b{ax}{nu}"]
        grads.update(extra)
    ts.synchronize()
    return J, traces, grads


class FdtdMisfit:
    """``torch.autograd.Function``: J(raw maps) with the engine's adjoint as backward."""

    @staticmethod
    def apply(template: DeviceInputs, observed, checkpoint_every: int, *maps):
        torch = _torch()

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, *tensors):
                inp = dataclasses.replace(template, maps={
                    **template.maps,
                    **{k: t.detach().to(torch.float32).contiguous()
                       for k, t in zip(RAW_MAPS, tensors)}})
                with Engine(inp, validate=False) as eng:
                    J, traces, grads = map_gradients(eng, observed, checkpoint_every)
                ctx.grads = [grads[k] for k in RAW_MAPS]
                ctx.dtypes = [t.dtype for t in tensors]
                ctx.traces = traces
                return torch.tensor(J, dtype=torch.float64, device=observed.device)

            @staticmethod
            def backward(ctx, gJ):
                return tuple((gJ * g).to(dt) for g, dt in zip(ctx.grads, ctx.dtypes))

        return _Fn.apply(*maps)


class AdjointProblem:
    """2D or 3D medium -> engine inputs, differentiable in c, rho and alpha0 (gamma held fixed).

    ``shape``: the medium's cells (depth first). The source is the whole plane (row in 2D) at
    depth ``source_row`` firing one pulse; sensors sit on the plane at depth ``sensor_row``, every
    ``sensor_step``-th cell along each lateral axis.
    """

    def __init__(self, shape, *, nt: int, f0: float = 3e6, ppw: int = 12, cfl: float = 0.2,
                 n_pml: int = 40, n_transition: int = 40, c_ref=None, device=None,
                 sensor_step: int = 1, source_row: int = 0, sensor_row: int = 5,
                 p0: float = 1e6, table=None):
        torch = _torch()
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.shape = tuple(shape)
        self.grid = Grid.from_cells(self.shape, f0=f0, nt=nt, ppw=ppw, cfl=cfl)
        self.nb = n_pml + n_transition + coefficients.N_TAPS
        self.n_pml, self.n_transition = n_pml, n_transition
        self.table = table or default_table()
        self.c_ref = c_ref   # starting medium: fixes dcmap/dmap
        self.source_row, self.sensor_row = source_row, sensor_row
        self.sensor_step = sensor_step
        self.p0 = p0

    def _relaxation(self, a0, gam):
        """Parameters linear in alpha0: d = alpha0 * d(1, gamma); rates from the gamma bin."""
        torch = _torch()
        t = self.table
        top = len(t.alpha_list) - 1
        pl = torch.as_tensor(t.power_list.round(10), device=gam.device)
        g = torch.clamp(gam, float(t.power_list.min()), float(t.power_list.max().round(4)))
        ig = torch.clamp(torch.searchsorted(pl, g.contiguous()), 0, len(pl) - 1)
        unit = torch.as_tensor(t.table[top] / max(float(t.alpha_list[top]), 1e-30),
                               device=gam.device)
        rates = torch.as_tensor(t.table[top], device=gam.device)
        keys = relaxation_param_keys(2)
        out = {}
        for i, k in enumerate(keys):
            if k.startswith("kappa"):
                out[k] = torch.ones_like(a0)
            elif k.startswith("d_"):
                out[k] = a0 * unit[ig, i]
            else:
                out[k] = rates[ig, i]
        return out

    def build(self, c, rho, a0, gam) -> DeviceInputs:
        """Engine inputs (maps keep the autograd graph of c, rho, a0)."""
        torch = _torch()
        nb, nd = self.nb, len(self.shape)
        p = self._relaxation(a0, gam)
        for op in ("x1", "x2"):  # mechanism sort by time constant (fullwave/medium.py:121-209)
            t1 = p[f"d_{op}_nu1"] / p[f"kappa_{op}"] + p[f"alpha_{op}_nu1"]
            t2 = p[f"d_{op}_nu2"] / p[f"kappa_{op}"] + p[f"alpha_{op}_nu2"]
            sw = (t2 < t1).detach()
            for var in ("d", "alpha"):
                a, b = p[f"{var}_{op}_nu1"], p[f"{var}_{op}_nu2"]
                p[f"{var}_{op}_nu1"], p[f"{var}_{op}_nu2"] = torch.where(sw, b, a), torch.where(sw, a, b)
        p = {k: extend_edge(v, nb) for k, v in p.items()}
        fw2 = pml_relaxation_maps_t({k: v.clone() for k, v in p.items()}, n_pml=self.n_pml,
                                    n_transition=self.n_transition, dt=self.grid.dt,
                                    c0=self.grid.c0, dx=self.grid.dx)
        ce, re = extend_edge(c, nb), extend_edge(rho, nb)
        maps = {"rho": re, "K": ce * ce * re, "kappau": fw2["kappa_u"], "kappax": fw2["kappa_x"]}
        for nu in (1, 2):
            for ax in ("u", "x"):
                maps[f"apml{ax}{nu}"] = fw2[f"a_pml_{ax}{nu}"]
                maps[f"bpml{ax}{nu}"] = fw2[f"b_pml_{ax}{nu}"]
        cref = extend_edge(self.c_ref if self.c_ref is not None else c.detach(), nb).detach()
        cmin, cmax = float(cref.min()), float(cref.max())
        dmap = coefficients.d_map(np.array([cmin, cmax]), self.grid.dt, self.grid.dx,
                                  is_3d=nd == 3)
        dcmap = (torch.round(cref + 1e-9) - round(cmin + 1e-9)).to(torch.int32).contiguous()
        sig = _pulse(self.grid, self.p0)

        def plane(row, step):   # (row, lateral...) coordinates of a depth plane, C order
            lat = np.meshgrid(*[np.arange(0, n, step) for n in self.shape[1:]], indexing="ij")
            lat = [a.reshape(-1) for a in lat]
            return np.stack([np.full(lat[0].size, row)] + lat, axis=1) + nb

        icc = plane(self.source_row, 1)
        outc = plane(self.sensor_row, self.sensor_step)
        dev = c.device
        i32 = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.int32), device=dev)  # noqa: E731
        fmaps = {k: v.detach().to(torch.float32).contiguous() for k, v in maps.items()}
        fmaps["c"] = ce.detach().to(torch.float32).contiguous()
        fmaps["beta"] = torch.zeros_like(fmaps["rho"])
        d = DeviceInputs(shape=tuple(n + 2 * nb for n in self.shape), nt=self.grid.nt,
                         spacing=(self.grid.dx,) * nd, dt=self.grid.dt, c0=self.grid.c0,
                         mod_t=1, d=coefficients.d_matrix(self.grid.cfl, is_3d=nd == 3),
                         dmap=dmap, dcmap=dcmap, maps=fmaps, icc=i32(icc),
                         icmat=torch.as_tensor(np.tile(sig, (len(icc), 1)), device=dev),
                         outc=i32(outc), icczero=i32(np.zeros((0, nd))))
        d.diff_maps = maps
        return d

    def misfit(self, c, rho, a0, gam, observed, checkpoint_every: int = 200):
        """J as a differentiable torch scalar of c, rho, a0."""
        d = self.build(c, rho, a0, gam)
        return FdtdMisfit.apply(d, observed, checkpoint_every,
                                *[d.diff_maps[k] for k in RAW_MAPS])


def _pulse(grid, p0):
    from .pulse import gaussian_modulated_sinusoidal_signal  # noqa: PLC0415

    return gaussian_modulated_sinusoidal_signal(nt=grid.nt, duration=grid.duration, ncycles=2,
                                                drop_off=2, f0=grid.f0, p0=p0).astype(np.float32)
