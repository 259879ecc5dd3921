"""Depth-slab decomposition of one simulation with a halo exchange every time step.

The reference splits the depth axis (x) of a simulation into contiguous slabs, one per GPU, and
exchanges slab halos inside its executables (README.md:249-261, "x ordering ... due to the
efficiency of the multiple-GPU execution"). This module is that decomposition for this engine:

* the body rows are split into contiguous owned ranges; each slab's grid is its owned rows plus
  ``overlap`` rows on each inner side (and the 8-row ghost layer beyond them), with its own maps,
  sources (every source inside its grid: the overlap is recomputed), air cells and the sensors of
  its owned rows only;
* every slab advances one time step; then each inner boundary copies the ``overlap`` rows of every
  state field from the slab that owns them. With ``overlap >= 15`` the owned rows of every slab
  stay exactly equal to the single-domain solve: one step spoils the 8 rows next to a slab's cut
  through the velocity stencil and 7 more through the pressure stencil, and those rows are then
  overwritten from their owner.

``exchange`` is pluggable: device-local copies between engine handles (``fw_copy_state_rows``,
:func:`run_slabs`), or any transport between processes (the gloo test runs the FP64 oracle per
rank and exchanges over ``torch.distributed``). On one GPU the slabs run one after the other;
the exchange protocol is what a multi-GPU run would use between peers.
"""

from __future__ import annotations

import dataclasses

import numpy as np

from . import coefficients

GHOST = coefficients.N_TAPS
OVERLAP = 16


@dataclasses.dataclass(frozen=True)
class Slab:
    own: tuple      # owned global body rows [o0, o1)
    dom: tuple      # global rows of the slab's grid [d0, d1)

    def local(self, row: int) -> int:
        return row - self.dom[0]


def slab_layout(nx: int, n_slabs: int, overlap: int = OVERLAP) -> list:
    """Owned ranges and grids of ``n_slabs`` depth slabs of an ``nx``-row grid."""
    if overlap < 15:
        raise ValueError("overlap must be at least 15 rows (velocity 8 + pressure 7)")
    body0, body1 = GHOST, nx - GHOST
    edges = np.linspace(body0, body1, n_slabs + 1).round().astype(int)
    slabs = []
    for s in range(n_slabs):
        o0, o1 = int(edges[s]), int(edges[s + 1])
        if o1 - o0 < overlap:
            raise ValueError(f"slab {s} owns {o1 - o0} rows, fewer than the overlap {overlap}")
        d0 = 0 if s == 0 else o0 - overlap - GHOST
        d1 = nx if s == n_slabs - 1 else o1 + overlap + GHOST
        slabs.append(Slab((o0, o1), (d0, d1)))
    return slabs


def exchanges(slabs: list, overlap: int = OVERLAP) -> list:
    """Row copies after every step: (dst slab, dst local row, src slab, src local row, rows)."""
    out = []
    for s in range(len(slabs) - 1):
        a, b = slabs[s], slabs[s + 1]
        cut = a.own[1]                      # == b.own[0]
        out.append((s, a.local(cut), s + 1, b.local(cut), overlap))                     # a <- b
        out.append((s + 1, b.local(cut - overlap), s, a.local(cut - overlap), overlap))  # b <- a
    return out


def slice_inputs(inp, slab: Slab):
    """Engine inputs of one slab and the global indices of the sensors it records."""
    d0, d1 = slab.dom
    o0, o1 = slab.own
    rows = lambda c: np.asarray(c)[:, 0]  # noqa: E731

    def keep(coords, lo, hi):
        c = np.asarray(coords)
        return (rows(c) >= lo) & (rows(c) < hi) if c.size else np.zeros(0, dtype=bool)

    def shift(coords, mask):
        c = np.array(np.asarray(coords)[mask], dtype=np.int32)
        if c.size:
            c[:, 0] -= d0
        return c

    src = keep(inp.icc, d0, d1)
    sen = keep(inp.outc, o0, o1)
    air = keep(inp.icczero, d0, d1)
    new = dataclasses.replace(
        inp,
        shape=(d1 - d0,) + tuple(inp.shape[1:]),
        maps={k: np.ascontiguousarray(np.asarray(v)[d0:d1]) for k, v in inp.maps.items()},
        dcmap=np.ascontiguousarray(np.asarray(inp.dcmap)[d0:d1]),
        icc=shift(inp.icc, src),
        icmat=np.ascontiguousarray(np.asarray(inp.icmat)[src]),
        outc=shift(inp.outc, sen),
        icczero=shift(inp.icczero, air).reshape(-1, len(inp.shape)),
    )
    return new, np.flatnonzero(sen)


def run_slabs(inp, n_slabs: int = 2, overlap: int = OVERLAP, stream=None) -> np.ndarray:
    """Full solve of ``inp`` as ``n_slabs`` depth slabs on the current GPU with a device-local
    halo exchange after every step; returns traces ``[n_out, ncoordsout]`` like ``Engine.run``."""
    from .engine import Engine  # noqa: PLC0415

    slabs = slab_layout(inp.shape[0], n_slabs, overlap)
    parts = [slice_inputs(inp, s) for s in slabs]
    engines = [Engine(p, validate=False) for p, _ in parts]
    plan = exchanges(slabs, overlap)
    try:
        for e in engines:
            e.reset(stream)
        for _ in range(inp.nt):
            for e in engines:
                e.advance(1, stream)
            for dst, drow, src, srow, n in plan:
                engines[dst].copy_state_rows_from(engines[src], srow, drow, n, stream)
        out = np.zeros((inp.n_out, np.asarray(inp.outc).shape[0]), dtype=np.float32)
        for e, (_, idx) in zip(engines, parts):
            if idx.size:
                out[:, idx] = e.read_traces()
        return out
    finally:
        for e in engines:
            e.close()
