"""Host-side pieces of the serving loop (no GPU): arrival process, latency summary per request
kind, and the device-memory estimate of a gradient request."""

import numpy as np
import pytest


def test_poisson_arrivals_seeded_and_bounded():
    from fullwave25_gb300.server import poisson_arrivals

    a = poisson_arrivals(20.0, 10.0, seed=0)
    b = poisson_arrivals(20.0, 10.0, seed=0)
    np.testing.assert_array_equal(a, b)
    assert (np.diff(a) > 0).all() and a[-1] < 10.0 and 120 < len(a) < 280


def test_summary_splits_latency_by_kind():
    from fullwave25_gb300.server import Request, summarize

    reqs = []
    for i in range(10):
        r = Request(rid=i, arrival=float(i), build=None, kind="gradient" if i % 5 == 0 else "forward")
        r.admitted, r.finished = r.arrival, r.arrival + (3.0 if r.kind == "gradient" else 1.0)
        reqs.append(r)
    s = summarize(reqs, 20.0)
    assert s["requests"] == 10 and s["sims_per_s"] == 0.5
    assert s["by_kind"]["gradient"]["requests"] == 2
    assert s["by_kind"]["gradient"]["latency_s"]["p50"] == 3.0
    assert s["by_kind"]["forward"]["latency_s"]["max"] == 1.0
    assert "by_kind" not in summarize(reqs[1:5], 4.0)


def test_gradient_memory_estimate_grows_with_grid_and_checkpoints():
    torch = pytest.importorskip("torch")
    from fullwave25_gb300.adjoint import AdjointProblem
    from fullwave25_gb300.server import GradientJob, engine_bytes

    def job(n, nt, k):
        p = AdjointProblem((n, n), nt=nt, device=torch.device("cpu"), sensor_step=2)
        return GradientJob(problem=p, start=(), observed=np.zeros((nt, n // 2), np.float32),
                           checkpoint_every=k)

    small, big = job(128, 600, 200), job(256, 600, 200)
    assert big.bytes_needed() > 1.5 * small.bytes_needed()
    # checkpoints (nt / K) and the segment store (K + 1) are both wavefield copies:
    # K = 25 keeps 24 + 26 copies, K = 10 keeps 60 + 11, K = 200 keeps 3 + 201
    b10, b25 = job(128, 600, 10).bytes_needed(), job(128, 600, 25).bytes_needed()
    assert b25 < b10 < small.bytes_needed()
    nb = small.problem.nb
    assert small.bytes_needed() > engine_bytes((128 + 2 * nb, 128 + 2 * nb), 600, 64)


def test_admission_rule():
    """FIFO head admission: memory budget (an oversized request only when nothing else runs),
    idle worker streams for gradient requests, and the cap on grid cells stepping together
    (the first forward request is always admitted)."""
    from fullwave25_gb300.server import Request, admissible

    fwd = Request(rid=0, arrival=0.0, build=None, bytes_needed=4, cells=10)
    grad = Request(rid=1, arrival=0.0, build=None, bytes_needed=4, kind="gradient")
    big = Request(rid=2, arrival=0.0, build=None, bytes_needed=100, cells=10)
    kw = dict(used=0, budget_bytes=10, busy=False, free_workers=1, cells_active=0,
              forward_active=False, max_active_cells=None)
    assert admissible(fwd, **kw) and admissible(grad, **kw)
    assert not admissible(fwd, **{**kw, "used": 8, "busy": True})        # over the budget
    assert admissible(big, **kw)                                          # alone: runs anyway
    assert not admissible(big, **{**kw, "busy": True})
    assert not admissible(grad, **{**kw, "free_workers": 0})              # no idle worker
    capped = {**kw, "max_active_cells": 15, "busy": True, "used": 4}
    assert admissible(fwd, **capped)                                      # nothing stepping yet
    assert not admissible(fwd, **{**capped, "cells_active": 10, "forward_active": True})
    assert admissible(fwd, **{**capped, "cells_active": 5, "forward_active": True})
    assert admissible(grad, **{**capped, "cells_active": 10, "forward_active": True})
