"""FP64 NumPy oracle of the Fullwave 2.5 isotropic two-mechanism FDTD time loop.

TEST INFRASTRUCTURE ONLY. Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline import this module, and only as the checker or as the timed CPU baseline; the product
path never calls it.

Parity status. The reference engine exists only as closed CUDA executables
(fullwave/solver/bins/gpu/{2d,3d}/num_relax=2/*), built for x86-64 hosts; it cannot be built
from source, cannot run in a container without a GPU, and cannot run on the aarch64 GB300 host.
So the time loop below is **parity unpinned** against the reference engine's output. What is
pinned: every input array it consumes equals the reference's own pre-processing (golden
fixtures generated by importing the reference's Python), and the stencil geometry is fixed by the
reference's own coefficient table (the consistency identity ``sum (2m-1) d[m,0] +
2 (ndim-1) d[1,1] = 1``, which holds only for the off-axis layout used here).

Scheme restated from these reference sources:
* PDE: ``nabla_1 p + rho dv/dt = 0``, ``nabla_2 . v + (1/K) dp/dt = 0`` (README.md:37-44).
* Staggered derivative with eight axial taps per side and one off-axis tap, per-cell tap set
  ``dmap[:, :, dcmap]`` (fullwave/solver/input_file_writer.py:183-559, :805-821):
      (Dx f)(i+1/2) = [ sum_m c_m (f[i+m] - f[i+1-m])
                        + c_o sum_{transverse t, s=+-1} (f[i+1, t+s] - f[i, t+s]) ] / dX
* Stretched coordinates with two relaxation memory variables per derivative direction
  (Komatitsch & Martin 2007 recursive convolution, as used at fullwave/medium.py:273-289 and
  fullwave/solver/pml_builder.py:794-810):
      psi_nu <- b_nu psi_nu + a_nu D f ;  D~ f = D f / kappa + psi_1 + psi_2
  with ``kappau/apmlu/bpmlu`` for the pressure gradient and ``kappax/apmlx/bpmlx`` for the
  velocity divergence (fullwave/medium.py:357-372); the anisotropic build reads one set per
  derivative axis: u/w/v for the gradient along x/y/z and x/y/z for the divergence
  (fullwave/medium.py:374-406, input_file_writer.py:592-620).
* Leapfrog: velocities then pressure each step; body region ``[8, n-8)`` on every axis (the
  8-cell ghost layer of pml_builder.py:270-276); ghost cells stay zero.
* Nonlinearity: ``p <- p - dT (K + 2 beta p) div`` (beta = 0 in every benchmark workload).
* Exponential-attenuation engine (maps ``a_exp`` instead of relaxation maps): no memory
  variables, ``kappa = 1``; after each field update the field is multiplied by ``a_exp``
  (``exp(-dt alpha c0 / 2)``, so the two updates of a step attenuate by ``exp(-dt alpha c0)``).
* Source: hard source ``p[icc[k]] = icmat[k, n]`` for ``n < nTic`` after the pressure update;
  air cells ``icczero`` forced to zero; sensors recorded after that whenever ``n % modT == 0``
  (fullwave/source.py:25-77, fullwave/sensor.py:24-50, input_file_writer.py:753-762).
"""

from __future__ import annotations

import numpy as np

GHOST = 8


class OracleState:
    """FP64 state of one simulation: ``p``, ``v[a]``, ``psi[a][nu]`` (gradient) and
    ``phi[a][nu]`` (divergence) memory variables, full-grid arrays."""

    def __init__(self, shape):
        nd = len(shape)
        self.p = np.zeros(shape)
        self.v = [np.zeros(shape) for _ in range(nd)]
        self.psi = [[np.zeros(shape), np.zeros(shape)] for _ in range(nd)]
        self.phi = [[np.zeros(shape), np.zeros(shape)] for _ in range(nd)]


def _body(shape, offset=None):
    """Slices of the body region shifted by ``offset`` cells per axis."""
    nd = len(shape)
    offset = offset or (0,) * nd
    return tuple(slice(GHOST + o, n - GHOST + o) for n, o in zip(shape, offset))


def _unit(nd, axis, s=1):
    o = [0] * nd
    o[axis] = s
    return o


def _add(a, b):
    return tuple(x + y for x, y in zip(a, b))


class Oracle:
    """FP64 time loop over an ``EngineInputs`` (float32 inputs promoted to float64)."""

    def __init__(self, inputs):
        inputs.validate()
        self.inp = inputs
        self.shape = tuple(inputs.shape)
        nd = self.nd = len(self.shape)
        f64 = lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)  # noqa: E731
        body = _body(self.shape)
        m = {k: f64(v)[body] for k, v in inputs.maps.items()}
        dmap = f64(inputs.dmap)
        dc = np.asarray(inputs.dcmap)[body]
        self.taps = [dmap[k, 0][dc] for k in range(1, 9)]      # c_1..c_8 per body cell
        self.tap_off = dmap[1, 1][dc]                          # off-axis tap per body cell
        self.h = [float(np.float32(s)) for s in inputs.spacing]
        self.dt = float(np.float32(inputs.dt))
        self.rdt_rho = self.dt / m["rho"]
        self.dt_k = self.dt * m["K"]
        self.beta2dt = 2.0 * self.dt * m["beta"]
        self.has_beta = bool(np.any(m["beta"] != 0))
        # exponential-attenuation engine: no relaxation maps; each field update is followed by
        # a multiplication with a_exp (fullwave/medium.py:1068-1090)
        self.a_exp = m.get("a_exp")
        if self.a_exp is not None:
            self.axis_u = self.axis_x = [None] * nd
            self._init_io(inputs)
            return
        self.inv_kappa_u = 1.0 / m["kappau"]
        self.inv_kappa_x = 1.0 / m["kappax"]
        self.au = (m["apmlu1"], m["apmlu2"])
        self.bu = (m["bpmlu1"], m["bpmlu2"])
        self.ax = (m["apmlx1"], m["apmlx2"])
        self.bx = (m["bpmlx1"], m["bpmlx2"])
        # per derivative axis (anisotropic build): gradient maps u/w/v, divergence maps x/y/z;
        # the isotropic build uses the u and x maps on every axis
        iso = "kappay" not in m
        gl, dl = ("u", "w", "v"), ("x", "y", "z")
        self.axis_u = [(1.0 / m[f"kappa{gl[a]}"], (m[f"apml{gl[a]}1"], m[f"apml{gl[a]}2"]),
                        (m[f"bpml{gl[a]}1"], m[f"bpml{gl[a]}2"])) if not iso else None
                       for a in range(nd)]
        self.axis_x = [(1.0 / m[f"kappa{dl[a]}"], (m[f"apml{dl[a]}1"], m[f"apml{dl[a]}2"]),
                        (m[f"bpml{dl[a]}1"], m[f"bpml{dl[a]}2"])) if not iso else None
                       for a in range(nd)]
        self._init_io(inputs)

    def _init_io(self, inputs):
        f64 = lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)  # noqa: E731
        lin = lambda c: (np.ravel_multi_index(tuple(np.asarray(c).T), self.shape)  # noqa: E731
                         if len(c) else np.zeros(0, np.int64))
        self.icc = lin(inputs.icc)
        self.icmat = f64(inputs.icmat)
        self.icczero = lin(inputs.icczero)
        self.outc = lin(inputs.outc)
        # duplicate source cells: the last listed source wins
        if self.icc.size:
            _, last = np.unique(self.icc[::-1], return_index=True)
            keep = np.sort(self.icc.size - 1 - last)
            self.src_keep = keep
        else:
            self.src_keep = np.zeros(0, np.int64)
        self.state = OracleState(self.shape)
        self.step_index = 0

    # -- derivative operators -----------------------------------------------------------------
    def grad(self, f, axis):
        """Staggered derivative of cell-centred ``f`` at ``+1/2`` along ``axis`` (body cells)."""
        sh, nd = self.shape, self.nd
        e = _unit(nd, axis)
        acc = np.zeros(tuple(n - 2 * GHOST for n in sh))
        for m in range(1, 9):
            acc += self.taps[m - 1] * (f[_body(sh, _unit(nd, axis, m))]
                                       - f[_body(sh, _unit(nd, axis, 1 - m))])
        off = np.zeros_like(acc)
        for b in range(nd):
            if b == axis:
                continue
            for s in (1, -1):
                t = _unit(nd, b, s)
                off += f[_body(sh, _add(e, t))] - f[_body(sh, t)]
        return (acc + self.tap_off * off) / self.h[axis]

    def div_component(self, g, axis):
        """Staggered derivative of ``+1/2``-staggered ``g`` back at cell centres (body cells)."""
        sh, nd = self.shape, self.nd
        e_m = _unit(nd, axis, -1)
        acc = np.zeros(tuple(n - 2 * GHOST for n in sh))
        for m in range(1, 9):
            acc += self.taps[m - 1] * (g[_body(sh, _unit(nd, axis, m - 1))]
                                       - g[_body(sh, _unit(nd, axis, -m))])
        off = np.zeros_like(acc)
        for b in range(nd):
            if b == axis:
                continue
            for s in (1, -1):
                t = _unit(nd, b, s)
                off += g[_body(sh, t)] - g[_body(sh, _add(e_m, t))]
        return (acc + self.tap_off * off) / self.h[axis]

    # -- one time step ------------------------------------------------------------------------
    def step(self, record=None):
        st, body, n = self.state, _body(self.shape), self.step_index
        if self.a_exp is not None:
            return self._step_exponential(record)
        for a in range(self.nd):
            ik, au, bu = self.axis_u[a] or (self.inv_kappa_u, self.au, self.bu)
            g = self.grad(st.p, a)
            for nu in range(2):
                st.psi[a][nu][body] = bu[nu] * st.psi[a][nu][body] + au[nu] * g
            st.v[a][body] -= self.rdt_rho * (g * ik + st.psi[a][0][body] + st.psi[a][1][body])
        div = np.zeros(tuple(k - 2 * GHOST for k in self.shape))
        for a in range(self.nd):
            ik, ax, bx = self.axis_x[a] or (self.inv_kappa_x, self.ax, self.bx)
            dv = self.div_component(st.v[a], a)
            for nu in range(2):
                st.phi[a][nu][body] = bx[nu] * st.phi[a][nu][body] + ax[nu] * dv
            div += dv * ik + st.phi[a][0][body] + st.phi[a][1][body]
        pb = st.p[body]
        if self.has_beta:
            st.p[body] = pb - (self.dt_k + self.beta2dt * pb) * div
        else:
            st.p[body] = pb - self.dt_k * div
        flat = st.p.reshape(-1)
        if n < self.icmat.shape[1] and self.src_keep.size:
            flat[self.icc[self.src_keep]] = self.icmat[self.src_keep, n]
        if self.icczero.size:
            flat[self.icczero] = 0.0
        if record is not None and n % self.inp.mod_t == 0:
            record[n // self.inp.mod_t] = flat[self.outc]
        self.step_index += 1

    def _step_exponential(self, record):
        """v <- a_exp (v - dt/rho D p);  p <- a_exp (p - dt (K + 2 beta p) sum_a D'_a v_a)."""
        st, body, n = self.state, _body(self.shape), self.step_index
        for a in range(self.nd):
            st.v[a][body] = self.a_exp * (st.v[a][body] - self.rdt_rho * self.grad(st.p, a))
        div = np.zeros(tuple(k - 2 * GHOST for k in self.shape))
        for a in range(self.nd):
            div += self.div_component(st.v[a], a)
        pb = st.p[body]
        coef = self.dt_k + self.beta2dt * pb if self.has_beta else self.dt_k
        st.p[body] = self.a_exp * (pb - coef * div)
        self._finish_step(record)

    def _finish_step(self, record):
        st, n = self.state, self.step_index
        flat = st.p.reshape(-1)
        if n < self.icmat.shape[1] and self.src_keep.size:
            flat[self.icc[self.src_keep]] = self.icmat[self.src_keep, n]
        if self.icczero.size:
            flat[self.icczero] = 0.0
        if record is not None and n % self.inp.mod_t == 0:
            record[n // self.inp.mod_t] = flat[self.outc]
        self.step_index += 1

    def run(self, n_steps=None):
        """Advance ``n_steps`` (default: all ``nT``) and return traces ``[n_out, ncoordsout]``."""
        n_steps = self.inp.nt if n_steps is None else n_steps
        out = np.zeros(((n_steps + self.inp.mod_t - 1) // self.inp.mod_t, self.outc.size))
        for _ in range(n_steps):
            self.step(out)
        return out


def run_oracle(inputs, n_steps=None) -> np.ndarray:
    """Forward solve; returns FP64 sensor traces ``[n_out, ncoordsout]`` (time-major, like genout)."""
    return Oracle(inputs).run(n_steps)


def rel_l2(a, b) -> float:
    """``||a - b|| / ||b||`` in FP64 (0 when both are zero)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    return float(num / den) if den > 0 else float(num)
