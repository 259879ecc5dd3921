"""Batched (group) engine on the GPU: many uneven 2D simulations stepped together give the same
traces as each simulation run alone (bitwise: same kernel bodies), and match the FP64 oracle
within 1e-4 relative L2."""

import numpy as np
import pytest

from fdtd_oracle import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.fixture(scope="module")
def instances(cuda):
    from fullwave25_gb300.workloads_batch import batch_instance

    return [batch_instance(i, scale=0.12, n_pml=10, n_transition=10) for i in range(6)]


def test_group_equals_individual_runs(engine_lib, cuda, instances):
    from fullwave25_gb300.engine import EngineGroup

    engines = [d.make_engine() for d in instances]
    alone = [e.run() for e in engines]
    assert len({d.nt for d in instances}) > 1 and len({d.shape for d in instances}) > 1
    with EngineGroup(engines) as grp:
        for _ in range(2):  # twice: the group resets its members
            grp.run()
            for a, t in zip(alone, grp.traces()):
                np.testing.assert_array_equal(a, t)
    for e in engines:
        e.close()


def test_whole_run_graph_equals_stepwise_blocks(engine_lib, cuda, instances):
    """fw_group_run replays the whole run (every member to its own nt) as one captured graph;
    with FWGB_GROUP_RUN_GRAPH=0 the same run is issued as blocks of 64-step graphs. Traces are
    bitwise equal, on repeated runs (the graph is reused) and after the member set changes (the
    graph is rebuilt)."""
    import os

    from fullwave25_gb300.engine import EngineGroup

    engines = [d.make_engine() for d in instances]
    os.environ["FWGB_GROUP_RUN_GRAPH"] = "0"
    try:
        with EngineGroup(engines) as grp:
            grp.run()
            blocks = grp.traces()
    finally:
        os.environ.pop("FWGB_GROUP_RUN_GRAPH", None)
    with EngineGroup(engines) as grp:
        for _ in range(2):
            grp.run()
            for a, t in zip(blocks, grp.traces()):
                np.testing.assert_array_equal(a, t)
        grp.set_members(engines[1:4])
        grp.run()
        for a, t in zip(blocks[1:4], grp.traces()):
            np.testing.assert_array_equal(a, t)
    for e in engines:
        e.close()


def test_group_member_matches_oracle(engine_lib, cuda, instances):
    from fdtd_oracle_c import run_oracle_c
    from fullwave25_gb300.engine import EngineGroup
    from fullwave25_gb300.workloads3d import to_host_inputs

    engines = [d.make_engine() for d in instances[:3]]
    with EngineGroup(engines) as grp:
        grp.run()
        got = grp.traces()
    for d, g in zip(instances[:3], got):
        err = rel_l2(g, run_oracle_c(to_host_inputs(d)))
        assert err < TOL, f"{d.spec}: rel-L2 {err:.3e}"
    for e in engines:
        e.close()


def test_group_rejects_3d_member(engine_lib, cuda):
    from fullwave25_gb300.engine import EngineError, EngineGroup
    from golden_io import load_case_inputs
    from fullwave25_gb300.engine import Engine

    with Engine(load_case_inputs("3d_small")) as e3:
        with pytest.raises(EngineError, match="FW_ERR_UNSUPPORTED"):
            EngineGroup([e3])


def _group(engines, **env):
    import os

    from fullwave25_gb300.engine import EngineGroup

    keys = ("FWGB_VARIANT", "FWGB_SHAPE2D", "FWGB_AUTOTUNE", "FWGB_STREAM2D")
    old = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ.pop(k, None)
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        return EngineGroup(engines)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


SHAPE_TILES = {0: (8, 32, 1), 1: (16, 64, 1), 2: (32, 64, 1), 3: (16, 128, 1), 4: (32, 128, 1),
               5: (64, 128, 1)}


@pytest.mark.parametrize("shape", sorted(SHAPE_TILES))
def test_group_every_kernel_shape_equals_alone(engine_lib, cuda, instances, shape):
    """Group row-march kernels (per-member TMA maps in global memory, staged argument blocks),
    with a beta/air member mixed in so the beta pressure kernel runs: bitwise equal to solo runs."""
    from fullwave25_gb300.engine import Engine
    from golden_io import load_case_inputs

    engines = [d.make_engine() for d in instances[:4]]
    engines.append(Engine(load_case_inputs("2d_air_beta"), validate=False))
    alone = [e.run() for e in engines]
    with _group(engines, FWGB_SHAPE2D=shape) as grp:
        assert grp.block_tile == SHAPE_TILES[shape]
        grp.run()
        for a, t in zip(alone, grp.traces()):
            np.testing.assert_array_equal(a, t)
    for e in engines:
        e.close()


@pytest.mark.parametrize("shape", [1, 2, 3, 4, 5])
def test_persistent_group_run_equals_alone(engine_lib, cuda, instances, shape):
    """FWGB_GROUP_PERSISTENT=1: the whole run of the group as one persistent cooperative launch
    (grid barriers between the phases, members leaving the work list at their own nt), with a
    beta/air member mixed in: bitwise equal to solo runs, on a repeated run and after the member
    set changes."""
    import os

    from fullwave25_gb300.engine import Engine
    from golden_io import load_case_inputs

    engines = [d.make_engine() for d in instances[:4]]
    engines.append(Engine(load_case_inputs("2d_air_beta"), validate=False))
    alone = [e.run() for e in engines]
    with _group(engines, FWGB_SHAPE2D=shape) as grp:
        os.environ["FWGB_GROUP_PERSISTENT"] = "1"
        try:
            for _ in range(2):
                grp.run()
                for a, t in zip(alone, grp.traces()):
                    np.testing.assert_array_equal(a, t)
            grp.set_members(engines[1:3])
            grp.run()
            for a, t in zip(alone[1:3], grp.traces()):
                np.testing.assert_array_equal(a, t)
        finally:
            os.environ.pop("FWGB_GROUP_PERSISTENT", None)
    for e in engines:
        e.close()


def test_group_register_loads_equal_streaming(engine_lib, cuda, instances):
    engines = [d.make_engine() for d in instances[:4]]
    alone = [e.run() for e in engines]
    with _group(engines, FWGB_SHAPE2D=1, FWGB_STREAM2D=0) as grp:
        grp.run()
        for a, t in zip(alone, grp.traces()):
            np.testing.assert_array_equal(a, t)
    for e in engines:
        e.close()


def test_group_autotune_keeps_results(engine_lib, cuda, instances):
    engines = [d.make_engine() for d in instances]
    alone = [e.run() for e in engines]
    with _group(engines) as grp:
        grp.run()                          # first run times every shape, then solves
        tile = grp.block_tile
        for a, t in zip(alone, grp.traces()):
            np.testing.assert_array_equal(a, t)
        grp.run()
        assert grp.block_tile == tile      # tuned once
        for a, t in zip(alone, grp.traces()):
            np.testing.assert_array_equal(a, t)
    for e in engines:
        e.close()


def test_host_api_instance_matches_device_built_instance(engine_lib, cuda):
    """The batched workload built on the device and the same instance built through the host-side
    API (NumPy medium, relaxation lookup, PML builder) give the same traces."""
    from fdtd_oracle import rel_l2
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads_batch import batch_inputs_host, batch_instance

    kw = dict(scale=0.12, n_pml=10, n_transition=10)
    for i in (0, 5):
        d = batch_instance(i, **kw)
        h = batch_inputs_host(i, **kw)
        assert tuple(h.shape) == tuple(d.shape) and h.nt == d.nt
        with d.make_engine() as a, Engine(h) as b:
            ta, tb = a.run(), b.run()
        assert np.abs(ta).max() > 0
        err = rel_l2(tb, ta)
        assert err < 1e-5, f"instance {i}: rel-L2 {err:.3e}"
