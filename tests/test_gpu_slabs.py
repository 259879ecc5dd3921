"""Depth-slab decomposition on one GPU (``-m gpu``): a simulation run as 2 or 3 depth slabs, each
its own engine handle, with the overlap rows of every state field copied between handles after
every step (fw_copy_state_rows), gives the single-domain traces bitwise."""

import numpy as np
import pytest

from golden_io import load_case_inputs

pytestmark = pytest.mark.gpu


def _plain2d():
    from fullwave25_gb300.workloads import plain_2d_inputs

    inp = plain_2d_inputs(shape=(96, 48), nt=150, n_pml=8, n_transition=8)
    nx, ny = inp.shape
    rng = np.random.default_rng(1)
    inp.outc = np.stack([np.arange(8, nx - 8), np.full(nx - 16, ny // 3)], 1).astype(np.int32)
    inp.icczero = np.stack([rng.integers(40, 80, 30), rng.integers(8, ny - 8, 30)], 1).astype(np.int32)
    return inp


def _volume3d():
    from fullwave25_gb300.workloads3d import plain_3d_device_inputs, to_host_inputs

    inp = to_host_inputs(plain_3d_device_inputs(shape=(48, 40, 72), nt=80, n_pml=8,
                                                n_transition=8, sensor_plane=24,
                                                element_height=8))
    nx = inp.shape[0]
    inp.outc = np.stack([np.arange(8, nx - 8), np.full(nx - 16, inp.shape[1] // 2),
                         np.full(nx - 16, inp.shape[2] // 2)], 1).astype(np.int32)
    return inp


@pytest.mark.parametrize("case,n_slabs", [("plain2d", 2), ("plain2d", 3), ("volume3d", 2)])
def test_slabs_equal_single_domain(engine_lib, cuda, case, n_slabs):
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.slabs import run_slabs

    inp = _plain2d() if case == "plain2d" else _volume3d()
    with Engine(inp) as e:
        ref = e.run()
    assert np.abs(ref).max() > 0
    got = run_slabs(inp, n_slabs)
    np.testing.assert_array_equal(got, ref)


def test_copy_rejects_mismatched_cross_sections(engine_lib, cuda):
    from fullwave25_gb300.engine import Engine, EngineError

    a = load_case_inputs("2d_small")
    b = load_case_inputs("3d_small")
    with Engine(a) as ea, Engine(b) as eb:
        with pytest.raises(EngineError, match="cross-section"):
            ea.copy_state_rows_from(eb, 8, 8, 4)
        with pytest.raises(EngineError, match="outside"):
            ea.copy_state_rows_from(ea, 0, a.shape[0] - 2, 4)
