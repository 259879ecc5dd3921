"""2D row-march kernels and the 2D kernel-shape autotuner (``-m gpu``).

Every 2D kernel shape (the direct kernels and the row-march blocks of TY columns x XC rows)
performs the same floating-point operations in the same order per cell, so traces must be
bit-identical across shapes; the oracle comparison of the default (autotuned) path keeps the
engine's usual 1e-4 relative-L2 bar against the FP64 oracle.
"""

import os

import numpy as np
import pytest

from fdtd_oracle import rel_l2
from golden_io import load_case_inputs

pytestmark = pytest.mark.gpu
TOL = 1e-4
MARCH_SHAPES = (1, 2, 3, 4, 5, 6, 7)   # march 1-5, persistent 6, TMA tiles 7; 0 = direct kernels
VARIANT = {1: "march", 2: "march", 3: "march", 4: "march", 5: "march", 6: "persistent",
           7: "tile"}


def _engine(inp, **env):
    from fullwave25_gb300.engine import Engine

    keys = ("FWGB_VARIANT", "FWGB_SHAPE2D", "FWGB_AUTOTUNE", "FWGB_STREAM2D")
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


def _scattered(inp, seed):
    """Sources, air cells and sensors spread over the whole grid, ghost cells included, so that
    every march block's list-tile rectangle (and the clamped edge tiles) carries entries."""
    rng = np.random.default_rng(seed)
    nx, ny = inp.shape
    pick = lambda n: np.stack([rng.integers(0, nx, n), rng.integers(0, ny, n)], 1).astype(np.int32)
    inp.icc = pick(300)
    inp.icmat = rng.standard_normal((300, inp.nt_ic)).astype(np.float32) * 1e3
    inp.outc = pick(400)
    inp.icczero = pick(500)
    return inp


@pytest.fixture(scope="module")
def ragged_2d(cuda):
    from fullwave25_gb300.workloads import plain_2d_inputs

    # extended grid 276 x 326: body 260 x 310, ragged for every shape along both axes
    return _scattered(plain_2d_inputs(shape=(100, 150), nt=300), seed=5)


@pytest.mark.parametrize("case", ["2d_small", "2d_air_beta", "2d_nopml", "2d_aniso", "2d_exp"])
def test_every_march_shape_equals_direct_bitwise(engine_lib, cuda, case):
    inp = load_case_inputs(case)
    with _engine(inp, FWGB_VARIANT="direct") as ed:
        ref = ed.run()
        assert ed.kernel_variant == "direct"
    assert np.abs(ref).max() > 0
    for k in MARCH_SHAPES:
        with _engine(inp, FWGB_SHAPE2D=k) as em:
            got = em.run()
            assert em.kernel_variant == VARIANT[k]
        np.testing.assert_array_equal(got, ref, err_msg=f"{case}: shape {k}")


def test_scattered_sources_air_sensors_every_shape(engine_lib, cuda, ragged_2d):
    with _engine(ragged_2d, FWGB_VARIANT="direct") as ed:
        ref = ed.run()
    assert np.abs(ref).max() > 0
    for k in MARCH_SHAPES:
        with _engine(ragged_2d, FWGB_SHAPE2D=k) as em:
            tile = em.block_tile
            got = em.run()
            pf = em.get_field(0)
        assert tile[1] % 32 == 0 and tile[0] % 8 == 0 and tile[2] == 1
        np.testing.assert_array_equal(got, ref, err_msg=f"shape {k}")
        # air cells are zero after the final step
        z = ragged_2d.icczero
        assert not pf[z[:, 0], z[:, 1]].any()


@pytest.mark.parametrize("case", ["ragged", "2d_air_beta"])
def test_register_and_streaming_row_march_equal(engine_lib, cuda, case, ragged_2d):
    """Row march with point-wise operands loaded by the threads (FWGB_STREAM2D=0) and staged by
    TMA (default for the isotropic engine): bitwise equal, every march shape."""
    inp = ragged_2d if case == "ragged" else load_case_inputs(case)
    for k in (1, 2, 3, 4, 5):
        with _engine(inp, FWGB_SHAPE2D=k) as es, _engine(inp, FWGB_SHAPE2D=k, FWGB_STREAM2D=0) as er:
            np.testing.assert_array_equal(es.run(), er.run(), err_msg=f"{case}: shape {k}")


def test_persistent_kernel_in_uneven_advances(engine_lib, cuda, ragged_2d):
    """The persistent kernel numbers its steps from the handle's step count: advancing in uneven
    pieces (and one step at a time) gives the traces of one full run."""
    with _engine(ragged_2d, FWGB_VARIANT="direct") as ed:
        ref = ed.run()
    with _engine(ragged_2d, FWGB_SHAPE2D=6) as e:
        e.reset()
        done = 0
        for n in (1, 1, 37, 100, 5):
            e.advance(n)
            done += n
        e.advance(ragged_2d.nt - done)
        assert e.current_step == ragged_2d.nt
        np.testing.assert_array_equal(e.read_traces(), ref)


def test_autotuned_engine_matches_direct_and_oracle(engine_lib, cuda, ragged_2d):
    from fdtd_oracle_c import run_oracle_c

    with _engine(ragged_2d, FWGB_VARIANT="direct") as ed:
        ref = ed.run()
    with _engine(ragged_2d) as ea:
        assert ea.block_tile == (8, 32, 1)         # direct until the first advance
        got = ea.run()
        chosen = ea.block_tile
        again = ea.run()                             # tuned once: no second round of trials
        assert ea.block_tile == chosen
    np.testing.assert_array_equal(got, ref)
    np.testing.assert_array_equal(again, ref)
    with _engine(ragged_2d) as eb:                   # same grid and physics: cached choice
        eb.run()
        assert eb.block_tile == chosen
    err = rel_l2(got, run_oracle_c(ragged_2d))
    assert err < TOL, f"rel-L2 {err:.3e}"


def test_autotune_disabled_and_short_runs_stay_direct(engine_lib, cuda, monkeypatch):
    inp = load_case_inputs("2d_small")
    monkeypatch.setenv("FWGB_AUTOTUNE", "0")   # read at the first advance
    with _engine(inp, FWGB_AUTOTUNE=0) as e:
        e.run()
        assert e.kernel_variant == "direct"
    monkeypatch.delenv("FWGB_AUTOTUNE")
    short = load_case_inputs("2d_small")          # fewer steps than two tuning trials
    short.nt = 100
    short.icmat = np.ascontiguousarray(short.icmat[:, :100])
    with _engine(short) as e:
        e.run()
        assert e.kernel_variant == "direct"


def test_invalid_shape_index_is_an_argument_error(engine_lib, cuda):
    from fullwave25_gb300.engine import EngineError

    with pytest.raises(EngineError, match="FWGB_SHAPE2D"):
        _engine(load_case_inputs("2d_small"), FWGB_SHAPE2D=17)


def test_wide_tap_table_every_shape(engine_lib, cuda):
    """Sound speeds spanning 1000-3000 m/s: 2001 tap sets, tap-set indices above 8 bits in the
    16-bit device map; every kernel shape equals the direct kernels and the FP64 oracle."""
    from fdtd_oracle_c import run_oracle_c
    from fullwave25_gb300 import coefficients
    from fullwave25_gb300.workloads import plain_2d_inputs

    inp = plain_2d_inputs(shape=(60, 70), nt=160, n_pml=8, n_transition=8)
    rng = np.random.default_rng(2)
    c = rng.uniform(1000.0, 3000.0, size=inp.shape).astype(np.float32)
    c[0, 0], c[-1, -1] = 1000.0, 3000.0
    inp.maps = dict(inp.maps)
    inp.maps["c"] = c
    inp.dmap = coefficients.d_map(c.astype(np.float64), inp.dt, inp.spacing[0], is_3d=False)
    inp.dcmap = coefficients.dc_map(c.astype(np.float64))
    assert inp.dmap.shape[2] == 2001 and inp.dcmap.max() == 2000
    with _engine(inp, FWGB_VARIANT="direct") as ed:
        ref = ed.run()
    assert np.abs(ref).max() > 0
    err = rel_l2(ref, run_oracle_c(inp))
    assert err < TOL, f"rel-L2 {err:.3e}"
    for k in MARCH_SHAPES:
        with _engine(inp, FWGB_SHAPE2D=k) as em:
            np.testing.assert_array_equal(em.run(), ref, err_msg=f"shape {k}")
