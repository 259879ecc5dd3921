"""Continuous-batching server: requests admitted while others run give the same traces as when
run alone (bitwise: same kernels), and latency statistics are reported."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(n, scale, rate_hz, seed=0):
    from fullwave25_gb300.server import Request, engine_bytes, poisson_arrivals
    from fullwave25_gb300.workloads_batch import batch_instance

    arrivals = poisson_arrivals(rate_hz, 10.0, seed)[:n]
    reqs = []
    for i, t in enumerate(arrivals):
        d = batch_instance(i, scale=scale, n_pml=10, n_transition=10)
        reqs.append(Request(rid=i, arrival=float(t), build=(lambda d=d: d),
                            bytes_needed=engine_bytes(d.shape, d.nt, d.outc.shape[0])))
    return reqs


def test_mixed_results_equal_alone(engine_lib, cuda):
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.server import serve_continuous

    reqs = _requests(10, 0.12, rate_hz=40.0)
    stats = serve_continuous(reqs, budget_bytes=4 << 30, chunk_steps=64)
    assert stats["requests"] == 10 and stats["chunks"] > 1
    assert all(r.finished >= r.arrival for r in reqs)
    for r in reqs:
        with Engine(r.build(), validate=False) as e:
            alone = e.run()
        np.testing.assert_array_equal(r.traces, alone)


def test_budget_limits_concurrency(engine_lib, cuda):
    from fullwave25_gb300.server import serve_continuous

    reqs = _requests(4, 0.12, rate_hz=1000.0)
    # a budget that fits one simulation at a time still completes every request
    stats = serve_continuous(reqs, budget_bytes=min(r.bytes_needed for r in reqs), chunk_steps=64)
    assert stats["requests"] == 4
    order = sorted(reqs, key=lambda r: r.admitted)
    for a, b in zip(order, order[1:]):
        assert b.admitted >= a.finished - 1e-9
