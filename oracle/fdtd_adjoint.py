"""FP64 NumPy adjoint of the oracle's time loop (2D and 3D).

TEST INFRASTRUCTURE ONLY: the reference adjoint that the GPU adjoint is checked against, itself
checked against central finite differences of the FP64 oracle (tests/test_adjoint_oracle.py).

Misfit ``J = 1/2 sum_{recorded n} || p^{n+1}[outc] - d_n ||^2`` of the sensor traces. The
gradient is taken with respect to the engine's per-cell coefficient maps (the float32 inputs the
time loop multiplies by): ``rdt_rho = dt/rho``, ``dt_k = dt K``, ``inv_ku = 1/kappau``,
``inv_kx = 1/kappax`` and the memory-variable coefficients ``au1 bu1 au2 bu2 ax1 bx1 ax2 bx2``.
The per-cell tap sets (``dcmap``) are piecewise constant in the sound speed and are held fixed.
Gradients with respect to physical maps (c, rho, alpha0) follow by the chain rule on the host.

Reverse of step n (state S_n before it, S_{n+1} after it):
  record:      lam_p[outc] += r_n              (r_n = traces_n - d_n)
  air, source: lam_p[icczero] = 0; lam_p[icc] = 0 (n < nTic)
  pressure:    d_a = D'_a v^{n+1/2};  L_nu = lam_phi_nu + (-k) lam_p
               lam_d_a = sum_nu ax_nu L_nu - k ikx lam_p ;  lam_phi_nu <- bx_nu L_nu
               grads: dt_k -= div lam_p;  inv_kx -= k lam_p sum_a d_a;
                      ax_nu += sum_a L_nu d_a;  bx_nu += sum_a L_nu phi_nu(S_n)
  velocity:    lam_v_a += D'_a^T lam_d_a;  g_a = D_a p^n;  M_nu = lam_psi_nu + (-r) lam_v_a
               lam_g_a = sum_nu au_nu M_nu - r iku lam_v_a ;  lam_psi_nu <- bu_nu M_nu
               grads: rdt_rho -= lam_v_a (iku g_a + psi_1' + psi_2');  inv_ku -= r g_a lam_v_a;
                      au_nu += M_nu g_a;  bu_nu += M_nu psi_nu(S_n)
  pressure at step start: lam_p += sum_a D_a^T lam_g_a

Nonlinear term (beta != 0): the pressure update is p' = p - (k + b p) div with b = 2 dt beta, so
k above becomes k + b p^n, lam_p passes to p^n times (1 - b div), and b gets the gradient
-p^n div lam_p (``beta2dt``).

Exponential-attenuation engine (maps ``rdt_rho``, ``dt_k``, ``a_exp``; forward
``v' = ae (v - r D_a p)``, ``p' = ae (p - k sum_a D'_a v'_a)``), reverse of step n:
  record, air, source as above
  pressure:    d = sum_a D'_a v'_a (S_{n+1});  lam_d = -ae k lam_p
               grads: dt_k -= ae d lam_p;  a_exp += lam_p (p^n - k d);  lam_p <- ae lam_p
  velocity:    lam_v_a += D'_a^T lam_d;  g_a = D_a p^n;  lam_g_a = -ae r lam_v_a
               grads: rdt_rho -= ae g_a lam_v_a;  a_exp += lam_v_a (v_a^n - r g_a);
               lam_v_a <- ae lam_v_a
  pressure at step start: lam_p += sum_a D_a^T lam_g_a
"""

from __future__ import annotations

import copy

import numpy as np

from fdtd_oracle import GHOST, Oracle, _body, _unit

GRAD_KEYS = ("rdt_rho", "dt_k", "inv_ku", "inv_kx", "au1", "bu1", "au2", "bu2",
             "ax1", "bx1", "ax2", "bx2")
EXP_GRAD_KEYS = ("rdt_rho", "dt_k", "a_exp")   # exponential-attenuation engine
GRAD_LETTERS = ("uwv", "xyz")   # per-axis map letters: pressure gradient, velocity divergence


def aniso_grad_keys(nd):
    """Gradient keys of the anisotropic engine: dt/rho, dt*K, then per derivative axis the five
    pressure-gradient maps (1/kappa, a1, b1, a2, b2 of u / w / v), then per axis the five
    velocity-divergence maps (of x / y / z) -- the order of the engine's gradient output."""
    keys = ["rdt_rho", "dt_k"]
    for letters in GRAD_LETTERS:
        for a in range(nd):
            g = letters[a]
            keys += [f"inv_k{g}", f"a{g}1", f"b{g}1", f"a{g}2", f"b{g}2"]
    return tuple(keys)


class AdjointOracle(Oracle):
    """FP64 forward (storing every state) and reverse pass."""

    def _taps_full(self):
        return self.taps, self.tap_off

    # transposes of the two derivative operators (scatter form over body cells)
    def grad_T(self, u, axis):
        """D_a^T u: u lives on body cells (the output of grad), result on the full grid."""
        sh, nd = self.shape, self.nd
        out = np.zeros(sh)
        e = _unit(nd, axis)
        w = u / self.h[axis]
        for m in range(1, 9):
            tw = self.taps[m - 1] * w
            out[_body(sh, _unit(nd, axis, m))] += tw
            out[_body(sh, _unit(nd, axis, 1 - m))] -= tw
        ow = self.tap_off * w
        for b in range(nd):
            if b == axis:
                continue
            for s in (1, -1):
                t = _unit(nd, b, s)
                out[_body(sh, tuple(x + y for x, y in zip(e, t)))] += ow
                out[_body(sh, t)] -= ow
        return out

    def div_T(self, u, axis):
        """D'_a^T u."""
        sh, nd = self.shape, self.nd
        out = np.zeros(sh)
        em = _unit(nd, axis, -1)
        w = u / self.h[axis]
        for m in range(1, 9):
            tw = self.taps[m - 1] * w
            out[_body(sh, _unit(nd, axis, m - 1))] += tw
            out[_body(sh, _unit(nd, axis, -m))] -= tw
        ow = self.tap_off * w
        for b in range(nd):
            if b == axis:
                continue
            for s in (1, -1):
                t = _unit(nd, b, s)
                out[_body(sh, t)] += ow
                out[_body(sh, tuple(x + y for x, y in zip(em, t)))] -= ow
        return out

    def forward_storing(self):
        """Run nT steps; returns (traces, states) with states[n] = state before step n."""
        states = []
        out = np.zeros((self.inp.n_out, self.outc.size))
        for _ in range(self.inp.nt):
            states.append(copy.deepcopy(self.state))
            self.step(out)
        states.append(copy.deepcopy(self.state))
        return out, states

    def _io_adjoint(self, lam_p, residual, n):
        """Record adjoint, air and source projections of step n on lam_p (in place)."""
        flat = lam_p.reshape(-1)
        if n % self.inp.mod_t == 0:
            np.add.at(flat, self.outc, residual[n // self.inp.mod_t])
        if self.icczero.size:
            flat[self.icczero] = 0.0
        if n < self.icmat.shape[1] and self.src_keep.size:
            flat[self.icc[self.src_keep]] = 0.0

    def adjoint_exponential(self, residual, states):
        """Reverse pass of the exponential-attenuation engine: FP64 body gradients with respect
        to ``rdt_rho``, ``dt_k`` and ``a_exp``."""
        nd, body = self.nd, _body(self.shape)
        bshape = tuple(k - 2 * GHOST for k in self.shape)
        keys = EXP_GRAD_KEYS + (("beta2dt",) if self.has_beta else ())
        G = {k: np.zeros(bshape) for k in keys}
        lam_p = np.zeros(self.shape)
        lam_v = [np.zeros(bshape) for _ in range(nd)]
        lam_g = None
        dtk, r, ae = self.dt_k, self.rdt_rho, self.a_exp
        for n in range(self.inp.nt - 1, -1, -1):
            Sn, Sn1 = states[n], states[n + 1]
            if lam_g is not None:
                for a in range(nd):
                    lam_p += self.grad_T(lam_g[a], a)
            self._io_adjoint(lam_p, residual, n)
            lp = lam_p[body].copy()
            d = np.zeros(bshape)
            for a in range(nd):
                d += self.div_component(Sn1.v[a], a)
            pn = Sn.p[body]
            k = dtk + self.beta2dt * pn if self.has_beta else dtk
            lam_d = -ae * k * lp
            G["dt_k"] -= ae * d * lp
            G["a_exp"] += lp * (pn - k * d)
            if self.has_beta:
                G["beta2dt"] -= ae * pn * d * lp
                lam_p[body] = ae * (1.0 - self.beta2dt * d) * lp
            else:
                lam_p[body] = ae * lp
            lam_g = []
            for a in range(nd):
                lv = lam_v[a] + self.div_T(lam_d, a)[body]
                g = self.grad(Sn.p, a)
                lam_g.append(-ae * r * lv)
                G["rdt_rho"] -= ae * g * lv
                G["a_exp"] += lv * (Sn.v[a][body] - r * g)
                lam_v[a] = ae * lv
        return G

    def adjoint(self, residual, states):
        """Reverse pass; ``residual`` [n_out, ncoordsout]. Returns dict of FP64 body gradients
        (``GRAD_KEYS``; ``EXP_GRAD_KEYS`` for the exponential-attenuation engine,
        ``aniso_grad_keys(nd)`` for the anisotropic one, whose maps differ per axis)."""
        if self.a_exp is not None:
            return self.adjoint_exponential(residual, states)
        nd, body = self.nd, _body(self.shape)
        bshape = tuple(k - 2 * GHOST for k in self.shape)
        aniso = self.axis_u[0] is not None
        keys = (aniso_grad_keys(nd) if aniso else GRAD_KEYS) + (("beta2dt",) if self.has_beta else ())
        G = {k: np.zeros(bshape) for k in keys}
        # per derivative axis: (1/kappa, (a1, a2), (b1, b2)) and the map letter of the keys
        U = [self.axis_u[a] or (self.inv_kappa_u, self.au, self.bu) for a in range(nd)]
        X = [self.axis_x[a] or (self.inv_kappa_x, self.ax, self.bx) for a in range(nd)]
        gu = [GRAD_LETTERS[0][a] if aniso else "u" for a in range(nd)]
        gx = [GRAD_LETTERS[1][a] if aniso else "x" for a in range(nd)]
        lam_p = np.zeros(self.shape)
        lam_v = [np.zeros(bshape) for _ in range(nd)]
        lam_psi = [[np.zeros(bshape), np.zeros(bshape)] for _ in range(nd)]
        lam_phi = [[np.zeros(bshape), np.zeros(bshape)] for _ in range(nd)]
        lam_g = None
        dtk, r = self.dt_k, self.rdt_rho
        for n in range(self.inp.nt - 1, -1, -1):
            Sn, Sn1 = states[n], states[n + 1]
            if lam_g is not None:
                for a in range(nd):
                    lam_p += self.grad_T(lam_g[a], a)
            self._io_adjoint(lam_p, residual, n)
            lp = lam_p[body].copy()
            pn = Sn.p[body]
            k = dtk + self.beta2dt * pn if self.has_beta else dtk   # coefficient of div
            # pressure step
            d = [self.div_component(Sn1.v[a], a) for a in range(nd)]
            div = np.zeros(bshape)
            for a in range(nd):
                div += d[a] * X[a][0] + Sn1.phi[a][0][body] + Sn1.phi[a][1][body]
            G["dt_k"] -= div * lp
            if self.has_beta:
                G["beta2dt"] -= pn * div * lp
                lam_p[body] = (1.0 - self.beta2dt * div) * lp
            lam_d = []
            for a in range(nd):
                ikx, ax, bx = X[a]
                L = [lam_phi[a][nu] - k * lp for nu in range(2)]
                lam_d.append(ax[0] * L[0] + ax[1] * L[1] - k * ikx * lp)
                G[f"inv_k{gx[a]}"] -= k * lp * d[a]
                for nu in range(2):
                    G[f"a{gx[a]}{nu + 1}"] += L[nu] * d[a]
                    G[f"b{gx[a]}{nu + 1}"] += L[nu] * Sn.phi[a][nu][body]
                    lam_phi[a][nu] = bx[nu] * L[nu]
            # velocity step
            lam_g = []
            for a in range(nd):
                iku, au, bu = U[a]
                lv = lam_v[a] + self.div_T(lam_d[a], a)[body]
                g = self.grad(Sn.p, a)
                M = [lam_psi[a][nu] - r * lv for nu in range(2)]
                lam_g.append(au[0] * M[0] + au[1] * M[1] - r * iku * lv)
                G["rdt_rho"] -= lv * (iku * g + Sn1.psi[a][0][body] + Sn1.psi[a][1][body])
                G[f"inv_k{gu[a]}"] -= r * g * lv
                for nu in range(2):
                    G[f"a{gu[a]}{nu + 1}"] += M[nu] * g
                    G[f"b{gu[a]}{nu + 1}"] += M[nu] * Sn.psi[a][nu][body]
                    lam_psi[a][nu] = bu[nu] * M[nu]
                lam_v[a] = lv
        return G


def misfit_and_gradient(inputs, observed):
    """J and its FP64 gradient w.r.t. the engine maps (body cells) for observed traces."""
    o = AdjointOracle(inputs)
    traces, states = o.forward_storing()
    res = traces - observed
    J = 0.5 * float(np.sum(res * res))
    return J, o.adjoint(res, states), traces


def misfit(inputs, observed, maps_override=None):
    """J with some engine maps replaced (FP64 arrays over body cells), for finite differences."""
    o = Oracle(inputs)
    if maps_override:
        for key, val in maps_override.items():
            attr = {"rdt_rho": "rdt_rho", "dt_k": "dt_k", "a_exp": "a_exp",
                    "beta2dt": "beta2dt"}.get(key)
            if o.axis_u[0] is not None and not attr:   # anisotropic: per-axis map sets
                letter = key[5] if key.startswith("inv_k") else key[1]
                side = 0 if letter in GRAD_LETTERS[0] else 1
                a = GRAD_LETTERS[side].index(letter)
                axes = o.axis_u if side == 0 else o.axis_x
                ik, aa, bb = axes[a]
                if key.startswith("inv_k"):
                    ik = val
                else:
                    pair = list(aa if key[0] == "a" else bb)
                    pair[int(key[2]) - 1] = val
                    aa, bb = (tuple(pair), bb) if key[0] == "a" else (aa, tuple(pair))
                axes[a] = (ik, aa, bb)
                continue
            attr = attr or {"inv_ku": "inv_kappa_u", "inv_kx": "inv_kappa_x"}.get(key)
            if attr:
                setattr(o, attr, val)
                if key == "beta2dt":
                    o.has_beta = True
            else:
                kind, nu = key[:2], int(key[2]) - 1
                tup = list(getattr(o, kind))
                tup[nu] = val
                setattr(o, kind, tuple(tup))
    traces = o.run()
    res = traces - observed
    return 0.5 * float(np.sum(res * res))
