"""3D plane march with TMA-staged point-wise operands (``-m gpu``).

The streaming kernels read every point-wise state field and map through 4D TMA boxes instead of
per-thread loads; the cell arithmetic is unchanged, so traces must be bit-identical to the
register-load plane march (FWGB_STREAM3D=0) and to the direct kernels, for either depth of the
point-wise ring, with and without the nonlinear (beta) term, on ragged grids with sources, air
cells and sensors anywhere; and within the engine's 1e-4 relative-L2 bar of the FP64 oracle.
"""

import os

import numpy as np
import pytest

from fdtd_oracle import rel_l2
from golden_io import load_case_inputs

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _engine(inp, **env):
    from fullwave25_gb300.engine import Engine

    keys = ("FWGB_VARIANT", "FWGB_STREAM3D", "FWGB_PS3D", "FWGB_XC3D")
    old = {k: os.environ.get(k) for k in keys}
    for k in keys:
        os.environ.pop(k, None)
    os.environ.update({k: str(v) for k, v in env.items()})
    try:
        return Engine(inp, validate=False)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _ragged_beta_3d():
    """The 3D golden case with a nonzero beta map, air cells and sources/sensors scattered over
    the whole grid (ghost cells included)."""
    inp = load_case_inputs("3d_small")
    rng = np.random.default_rng(7)
    shape = inp.shape
    inp.maps = dict(inp.maps)
    inp.maps["beta"] = (rng.random(shape) * 5.0).astype(np.float32)
    pick = lambda n: np.stack([rng.integers(0, s, n) for s in shape], 1).astype(np.int32)  # noqa: E731
    inp.icc = pick(200)
    inp.icmat = rng.standard_normal((200, inp.nt_ic)).astype(np.float32) * 1e3
    inp.outc = pick(300)
    inp.icczero = pick(150)
    return inp


CASES = {"3d_small": lambda: load_case_inputs("3d_small"), "ragged_beta": _ragged_beta_3d}


@pytest.mark.parametrize("case", sorted(CASES))
def test_stream_equals_register_march_and_direct(engine_lib, cuda, case):
    inp = CASES[case]()
    with _engine(inp, FWGB_VARIANT="direct") as ed:
        ref = ed.run()
    assert np.abs(ref).max() > 0
    with _engine(inp, FWGB_STREAM3D=0) as er:
        assert er.kernel_variant == "march"
        np.testing.assert_array_equal(er.run(), ref)
    for env in ({}, {"FWGB_XC3D": 64}, {"FWGB_PS3D": 3}):
        with _engine(inp, **env) as es:
            assert es.kernel_variant == "stream"
            np.testing.assert_array_equal(es.run(), ref, err_msg=f"{case}: {env}")


def test_stream_with_beta_matches_oracle(engine_lib, cuda):
    from fdtd_oracle_c import run_oracle_c

    inp = _ragged_beta_3d()
    with _engine(inp) as e:
        got = e.run()
        p = e.get_field(0)
    err = rel_l2(got, run_oracle_c(inp))
    assert err < TOL, f"rel-L2 {err:.3e}"
    z = inp.icczero
    assert not p[z[:, 0], z[:, 1], z[:, 2]].any()


def test_plain_3d_reduced_stream_vs_register(engine_lib, cuda):
    """Device-built plain 3D workload (multi-chunk march in x, 64-element source, sensor plane)."""
    from fullwave25_gb300.workloads3d import plain_3d_device_inputs

    d = plain_3d_device_inputs(shape=(160, 40, 72), nt=200, n_pml=8, n_transition=8,
                               sensor_plane=24, element_height=8)
    with _engine(d) as es, _engine(d, FWGB_STREAM3D=0) as er, _engine(d, FWGB_XC3D=64) as e8:
        assert es.kernel_variant == "stream" and es.block_tile[0] == 32
        assert e8.block_tile[0] == 64
        ref = er.run()
        np.testing.assert_array_equal(es.run(), ref)
        np.testing.assert_array_equal(e8.run(), ref)
