"""Serving loop: continuous batching of forward solves on one GPU.

Requests arrive over time (a seeded Poisson process in the benchmark). The loop admits arrived
requests in FIFO order while their device memory fits a budget, builds their media on the device,
and steps every admitted simulation together through the group engine (one launch per phase per
step over all their tiles). Between blocks of steps it retires finished simulations (their traces
are read back and their memory freed) and admits newly arrived ones, so a request never waits for
an unrelated long simulation to finish. Media and wavefields stay resident on the GPU for the life
of a request. ``serve_fifo`` is the one-at-a-time baseline on the same requests.
"""

from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .engine import Engine, EngineGroup


@dataclass
class Request:
    rid: int
    arrival: float                     # seconds after the stream starts
    build: object                      # callable -> DeviceInputs (built on the device)
    bytes_needed: int = 0
    kind: str = "forward"
    # filled by the server
    admitted: float = -1.0
    finished: float = -1.0
    traces: np.ndarray = field(default=None, repr=False)

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


def serve_continuous(requests, *, budget_bytes: int, chunk_steps: int = 256, stream=None,
                     clock=time.perf_counter) -> dict:
    """Run ``requests`` (sorted by arrival) with continuous batching; returns summary stats."""
    import torch  # noqa: PLC0415

    pending = sorted(requests, key=lambda r: r.arrival)
    active: list = []            # (request, engine)
    used = 0
    group = None
    t0 = clock()
    n_chunks = 0
    while pending or active:
        now = clock() - t0
        # admit arrived requests in FIFO order while the memory budget allows
        while pending and pending[0].arrival <= now and (
                used + pending[0].bytes_needed <= budget_bytes or not active):
            r = pending.pop(0)
            eng = Engine(r.build(), validate=False)
            r.admitted = clock() - t0
            active.append((r, eng))
            used += r.bytes_needed
        if not active:
            # idle until the next arrival
            wait = pending[0].arrival - (clock() - t0)
            if wait > 0:
                time.sleep(min(wait, 0.05))
            continue
        engines = [e for _, e in active]
        if group is None:
            group = EngineGroup(engines)
        else:
            group.set_members(engines)
        group.advance(chunk_steps, stream)
        torch.cuda.synchronize()
        n_chunks += 1
        still = []
        for r, e in active:
            if e.current_step >= e.inputs.nt:
                r.traces = e.read_traces()
                r.finished = clock() - t0
                used -= r.bytes_needed
                e.close()
            else:
                still.append((r, e))
        active = still
        if not active and group is not None:
            group.set_members([])
    if group is not None:
        group.close()
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
        with Engine(r.build(), validate=False) as eng:
            r.traces = eng.run()
        torch.cuda.synchronize()
        r.finished = clock() - t0
    return summarize(requests, clock() - t0)


def summarize(requests, wall_s: float, extra=None) -> dict:
    lat = np.array([r.latency for r in requests])
    out = {"requests": len(requests), "wall_s": wall_s, "sims_per_s": len(requests) / wall_s,
           "latency_s": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                         "p99": float(np.percentile(lat, 99)), "max": float(lat.max())}}
    if extra:
        out.update(extra)
    return out
