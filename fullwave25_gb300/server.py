"""Serving loop: continuous batching of forward and gradient solves on one GPU.

Requests arrive over time (a seeded Poisson process in the benchmark). The loop admits arrived
requests in FIFO order while their device memory fits a budget. Forward requests have their media
built on the device and are stepped together through the group engine (one launch per phase per
step over all their tiles, on the server's own stream); between blocks of steps the loop retires
finished simulations (traces read back, memory freed) and admits newly arrived ones, so a request
never waits for an unrelated long simulation to finish. Gradient requests (checkpointed forward +
discrete adjoint) run on worker threads, each on its own CUDA stream, so their kernels overlap
the group's on the device. Media and wavefields stay resident on the GPU for the life of a
request. ``serve_fifo`` is the one-at-a-time baseline on the same requests.
"""

from __future__ import annotations

import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

from .engine import Engine, EngineGroup


@dataclass
class GradientJob:
    """A gradient request: misfit of the starting medium against observed traces and its
    gradient with respect to the engine's coefficient maps (see :mod:`fullwave25_gb300.adjoint`)."""

    problem: object                    # AdjointProblem (grid, source, sensors, PML)
    start: tuple                       # (c, rho, alpha0, gamma) device tensors, original grid
    observed: object                   # device float32 [n_out, n_sensors]
    checkpoint_every: int = 200

    def bytes_needed(self) -> int:
        nb = self.problem.nb
        shape = tuple(s + 2 * nb for s in self.problem.shape)
        pitch = -(-shape[-1] // 32) * 32
        cells = shape[0] * pitch
        nt = self.problem.grid.nt
        # checkpoints plus two stores of checkpoint_every + 1 states (the next segment is
        # recomputed into one while the other is reversed)
        n_states = nt // self.checkpoint_every + 2 * (self.checkpoint_every + 1)
        fwd = engine_bytes(shape, nt, self.observed.shape[1])
        return fwd + cells * 4 * (11 * n_states + 15) + cells * 8 * 24

    def run(self, stream=None) -> dict:
        """Build the engine inputs on the device and evaluate J and the map gradients on
        ``stream`` (a torch stream, or None for the current one)."""
        import torch  # noqa: PLC0415

        from .adjoint import map_gradients  # noqa: PLC0415

        s = stream or torch.cuda.current_stream()
        with torch.cuda.stream(s):
            d = self.problem.build(*self.start)
            with Engine(d, validate=False) as eng:
                J, traces, grads = map_gradients(eng, self.observed, self.checkpoint_every, s)
        return {"J": J, "grads": grads}


@dataclass
class Request:
    rid: int
    arrival: float                     # seconds after the stream starts
    build: object                      # callable -> DeviceInputs (forward) or GradientJob
    bytes_needed: int = 0
    kind: str = "forward"              # "forward" or "gradient"
    cells: int = 0                     # grid cells (forward requests; 0 = not counted)
    # filled by the server
    admitted: float = -1.0
    finished: float = -1.0
    traces: np.ndarray = field(default=None, repr=False)
    result: dict = field(default=None, repr=False)   # gradient requests: {"J", "grads"}

    @property
    def latency(self) -> float:
        return self.finished - self.arrival


def engine_bytes(shape, nt, n_sensors, ndim=2) -> int:
    """Device bytes of one simulation: padded state + maps + dcmap + traces (+ lists, small)."""
    pitch = -(-shape[-1] // 32) * 32
    cells = int(np.prod(shape[:-1])) * pitch
    n_state = 1 + ndim + 4 * ndim
    return cells * 4 * (n_state + 13 + 1) + nt * n_sensors * 4


def poisson_arrivals(rate_hz: float, duration_s: float, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate_hz)
        if t >= duration_s:
            return np.array(out)
        out.append(t)


def admissible(r, *, used: int, budget_bytes: int, busy: bool, free_workers: int,
               cells_active: int, forward_active: bool, max_active_cells: int | None) -> bool:
    """Whether arrived request ``r`` (the head of the FIFO queue) may start now.

    ``used``: device bytes held by admitted requests; ``busy``: anything admitted and unfinished
    (a request larger than the whole budget runs only when nothing else does);
    ``free_workers``: idle gradient worker streams; ``cells_active`` / ``forward_active``: grid
    cells and presence of forward requests in (or joining) the group."""
    if used + r.bytes_needed > budget_bytes and busy:
        return False
    if r.kind == "gradient":
        return free_workers > 0
    return not (max_active_cells is not None and forward_active
                and cells_active + r.cells > max_active_cells)


def serve_continuous(requests, *, budget_bytes: int, chunk_steps: int = 256, stream=None,
                     clock=time.perf_counter, gradient_workers: int = 2,
                     max_active_cells: int | None = None) -> dict:
    """Run ``requests`` with continuous batching; returns summary stats.

    Forward requests are built on their own stream while the group runs a block and join the
    group engine between blocks of ``chunk_steps`` steps; gradient
    requests run on up to ``gradient_workers`` threads with a CUDA stream each. Admission is FIFO
    by arrival while the device-memory budget allows (a request larger than the budget runs
    alone) and, with ``max_active_cells``, while the group's forward requests hold at most that
    many grid cells: enough to keep the GPU's bandwidth busy, few enough that an overloaded
    stream does not share the GPU among every waiting request (which delays them all alike) but
    finishes the earlier arrivals first."""
    import torch  # noqa: PLC0415

    pending = sorted(requests, key=lambda r: r.arrival)
    active: list = []            # (request, engine) of admitted forward requests
    running: dict = {}           # future -> request, admitted gradient requests
    lock = threading.Lock()
    used = 0
    cells_active = 0
    group = None
    main = stream or torch.cuda.Stream()
    streams = [torch.cuda.Stream() for _ in range(max(1, gradient_workers))]
    free_streams = list(streams)
    pool = ThreadPoolExecutor(max_workers=max(1, gradient_workers))
    t0 = clock()
    n_chunks = 0

    def gradient(r, s):
        try:
            r.result = r.build().run(s)
            s.synchronize()
        finally:
            r.finished = clock() - t0

    build = torch.cuda.Stream()   # forward requests are built here, overlapping the group's steps
    joining: list = []            # built forward requests that join the group at the next block

    def admit():
        """Admit arrived requests in FIFO order while the memory budget (and the cell cap)
        allow: gradient requests start on a worker stream, forward requests are built."""
        nonlocal used, cells_active
        now = clock() - t0
        while pending and pending[0].arrival <= now and admissible(
                pending[0], used=used, budget_bytes=budget_bytes,
                busy=bool(active or joining or running), free_workers=len(free_streams),
                cells_active=cells_active, forward_active=bool(active or joining),
                max_active_cells=max_active_cells):
            r = pending.pop(0)
            if r.kind == "gradient":
                r.admitted = clock() - t0
                s = free_streams.pop()
                running[pool.submit(gradient, r, s)] = (r, s)
            else:
                cells_active += r.cells
                with torch.cuda.stream(build):
                    eng = Engine(r.build(), validate=False)
                r.admitted = clock() - t0
                joining.append((r, eng))
            used += r.bytes_needed

    try:
        while pending or active or joining or running:
            admit()
            # retire finished gradient requests
            for fut in [f for f in running if f.done()]:
                r, s = running.pop(fut)
                fut.result()  # re-raise a worker's error here
                free_streams.append(s)
                used -= r.bytes_needed
            active += joining
            joining = []
            if not active:
                # idle until the next arrival or a gradient finishes
                wait = (pending[0].arrival - (clock() - t0)) if pending else 0.01
                if wait > 0:
                    time.sleep(min(wait, 0.01))
                continue
            engines = [e for _, e in active]
            if group is None:
                group = EngineGroup(engines)
            else:
                group.set_members(engines)
            group.advance(chunk_steps, main.cuda_stream)
            admit()            # requests arriving meanwhile are built while the block runs
            main.synchronize()
            n_chunks += 1
            still = []
            for r, e in active:
                if e.current_step >= e.inputs.nt:
                    r.traces = e.read_traces(stream=main.cuda_stream)
                    r.finished = clock() - t0
                    used -= r.bytes_needed
                    cells_active -= r.cells
                    e.close()
                else:
                    still.append((r, e))
            active = still
            if not active and not joining and group is not None:
                group.set_members([])
    finally:
        # on an error (a worker's exception re-raised above, a failed build) release every
        # engine still held; on success all of them are closed already
        pool.shutdown(wait=True)
        if group is not None:
            group.close()
        for _, e in active + joining:
            e.close()
    del lock
    return summarize(requests, clock() - t0, extra={"chunks": n_chunks})


def serve_fifo(requests, *, clock=time.perf_counter) -> dict:
    """One-at-a-time FIFO baseline: each request runs alone after the previous one finished."""
    import torch  # noqa: PLC0415

    t0 = clock()
    for r in sorted(requests, key=lambda r: r.arrival):
        now = clock() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        r.admitted = clock() - t0
        if r.kind == "gradient":
            r.result = r.build().run()
        else:
            with Engine(r.build(), validate=False) as eng:
                r.traces = eng.run()
        torch.cuda.synchronize()
        r.finished = clock() - t0
    return summarize(requests, clock() - t0)


def summarize(requests, wall_s: float, extra=None) -> dict:
    def stats(rs):
        lat = np.array([r.latency for r in rs])
        return {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                "p99": float(np.percentile(lat, 99)), "max": float(lat.max())}

    out = {"requests": len(requests), "wall_s": wall_s, "sims_per_s": len(requests) / wall_s,
           "latency_s": stats(requests)}
    kinds = sorted({r.kind for r in requests})
    if len(kinds) > 1:
        out["by_kind"] = {k: {"requests": sum(r.kind == k for r in requests),
                              "latency_s": stats([r for r in requests if r.kind == k])}
                          for k in kinds}
    if extra:
        out.update(extra)
    return out
