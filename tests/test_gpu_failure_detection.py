"""Failure detection without a GPU fault (``-m gpu``): every spin-wait in the engine's kernels
is bounded. A self-test kernel waits on an mbarrier that nothing completes and another on a grid
barrier that counts a block that does not exist; each must give up after its limit, record it in
its status word and return, leaving the context usable."""

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_waits_give_up_and_report(engine_lib, cuda):
    from fullwave25_gb300.engine import selftest_waits

    t0 = time.perf_counter()
    mbar_status, barrier_status = selftest_waits()
    elapsed = time.perf_counter() - t0
    assert mbar_status & 0x1, hex(mbar_status)
    assert barrier_status & 0x4, hex(barrier_status)
    assert elapsed < 10.0


def test_context_usable_after_timeouts(engine_lib, cuda):
    from fullwave25_gb300.engine import Engine, selftest_waits
    from golden_io import load_case_inputs

    selftest_waits()
    inp = load_case_inputs("2d_small")
    with Engine(inp) as e:
        a = e.run()
    with Engine(inp) as e:
        np.testing.assert_array_equal(e.run(), a)
