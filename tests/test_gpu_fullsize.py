"""The benchmark configurations at their stated sizes against the FP64 C oracle (``-m gpu``).

Tolerance: sensor traces within 1e-4 relative L2 of the FP64 oracle, as in every parity test.
* plain 2D forward in full: 768 x 512 + PML 40 + transition 40 (944 x 688 extended cells),
  4000 time steps, 512 sensors;
* the largest member of the 64-simulation batch: instance 13, 2048 x 1536 + 176 (2224 x 1712
  extended cells, 3.8 M cells), with its nt of 8000 truncated to the first 1500 steps (the FP64
  oracle at 8000 steps would take minutes of host time);
* a block of the plain 3D medium larger than the benchmark's CPU sample: 64^3 + PML 16 +
  transition 16 (144^3 extended cells), the full 3000 time steps, a 32 x 32 sensor plane.
The oracle runs on every host core (OpenMP).
"""

import numpy as np
import pytest

from fdtd_oracle import rel_l2
from fdtd_oracle_c import OracleC, run_oracle_c

pytestmark = pytest.mark.gpu
TOL = 1e-4


def test_plain_2d_full_size_matches_oracle(engine_lib, cuda):
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads import plain_2d_inputs

    inp = plain_2d_inputs()
    assert tuple(inp.shape) == (944, 688) and inp.nt == 4000 and inp.outc.shape[0] == 512
    with Engine(inp) as eng:
        got = eng.run()
    ref = run_oracle_c(inp)
    assert got.shape == ref.shape == (4000, 512)
    err = rel_l2(got, ref)
    assert err < TOL, f"plain 2D 944 x 688 x 4000: rel-L2 {err:.3e}"


def test_largest_batch_member_matches_oracle(engine_lib, cuda):
    from fullwave25_gb300.workloads3d import to_host_inputs
    from fullwave25_gb300.workloads_batch import batch_instance

    n_steps = 1500
    d = batch_instance(13)
    assert tuple(d.shape) == (2224, 1712) and d.nt == 8000
    eng = d.make_engine()
    try:
        eng.advance(n_steps)
        got = eng.read_traces(0, n_steps)
    finally:
        eng.close()
    host = to_host_inputs(d)
    del d
    o = OracleC(host)
    try:
        ref = o.run(n_steps)
    finally:
        o.close()
    assert np.abs(ref).max() > 0
    err = rel_l2(got, ref)
    assert err < TOL, f"batch instance 13, first {n_steps} steps: rel-L2 {err:.3e}"


def test_plain_3d_block_full_nt_matches_oracle(engine_lib, cuda):
    from fullwave25_gb300.workloads3d import plain_3d_device_inputs, to_host_inputs

    d = plain_3d_device_inputs(shape=(64, 64, 64), nt=3000, n_pml=16, n_transition=16,
                               sensor_plane=32, element_height=16)
    assert tuple(d.shape) == (144, 144, 144)
    eng = d.make_engine()
    try:
        got = eng.run()
    finally:
        eng.close()
    ref = run_oracle_c(to_host_inputs(d))
    assert got.shape == ref.shape == (3000, 1024)
    err = rel_l2(got, ref)
    assert err < TOL, f"plain 3D 144^3 x 3000: rel-L2 {err:.3e}"
