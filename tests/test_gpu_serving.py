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


def test_cell_cap_limits_the_group(engine_lib, cuda):
    """With max_active_cells, the forward requests stepping together never hold more grid cells
    than the cap (unless one request alone exceeds it), and results still equal the alone runs."""
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.server import serve_continuous

    reqs = _requests(8, 0.12, rate_hz=1000.0)
    for r in reqs:
        r.cells = int(np.prod(r.build().shape))
    cap = 2 * int(np.median([r.cells for r in reqs]))
    stats = serve_continuous(reqs, budget_bytes=8 << 30, chunk_steps=64, max_active_cells=cap)
    assert stats["requests"] == 8
    most = 0
    for r in reqs:
        live = [q for q in reqs if q.admitted <= r.admitted < q.finished]
        most = max(most, len(live))
        assert len(live) == 1 or sum(q.cells for q in live) <= cap
    assert most >= 2   # the cap still lets requests share the group
    for r in reqs:
        with Engine(r.build(), validate=False) as e:
            np.testing.assert_array_equal(r.traces, e.run())


def test_forward_and_gradient_mix_equal_alone(engine_lib, cuda):
    """Gradient requests run on worker streams while forward requests step in the group: every
    forward result and every gradient equals the one computed alone."""
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.server import Request, serve_continuous
    from fullwave25_gb300.workloads_batch import gradient_job

    reqs = _requests(6, 0.12, rate_hz=40.0)
    jobs = [gradient_job(i, scale=0.12) for i in range(3)]
    for k, j in enumerate(jobs):
        reqs.append(Request(rid=100 + k, arrival=0.02 * k, build=(lambda j=j: j),
                            kind="gradient", bytes_needed=j.bytes_needed()))
    stats = serve_continuous(reqs, budget_bytes=8 << 30, chunk_steps=64, gradient_workers=2)
    assert stats["requests"] == 9 and set(stats["by_kind"]) == {"forward", "gradient"}
    for r in reqs:
        assert r.finished >= r.admitted >= r.arrival - 1e-9
        if r.kind == "forward":
            with Engine(r.build(), validate=False) as e:
                np.testing.assert_array_equal(r.traces, e.run())
        else:
            alone = r.build().run()
            assert r.result["J"] == alone["J"] and alone["J"] > 0
            for k, g in alone["grads"].items():
                np.testing.assert_allclose(r.result["grads"][k].cpu().numpy(), g.cpu().numpy(),
                                           rtol=1e-12, atol=0, err_msg=k)
