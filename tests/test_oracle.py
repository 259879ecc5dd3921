"""The FP64 oracle: committed traces, and physical/structural properties on CPU."""

import numpy as np
import pytest

from fdtd_oracle import Oracle, rel_l2, run_oracle
from golden_io import CASE_NAMES, HERE, load_case_inputs

TRACES = np.load(HERE / "oracle_traces.npz")


@pytest.mark.parametrize("name", CASE_NAMES)
def test_oracle_reproduces_committed_traces(name):
    out = run_oracle(load_case_inputs(name))
    np.testing.assert_allclose(out, TRACES[name], rtol=0, atol=1e-9 * np.abs(TRACES[name]).max())


def test_linearity_without_beta():
    inp = load_case_inputs("2d_small")
    a = run_oracle(inp, 80)
    inp.icmat = (2.5 * inp.icmat.astype(np.float64)).astype(np.float32)
    b = run_oracle(inp, 80)
    assert rel_l2(b, 2.5 * a) < 1e-6


def test_time_shift_invariance():
    inp = load_case_inputs("2d_small")
    a = run_oracle(inp, 120)
    shift = 7
    sh = np.zeros_like(inp.icmat)
    sh[:, shift:] = inp.icmat[:, :-shift]
    inp.icmat = sh
    b = run_oracle(inp, 120)
    np.testing.assert_allclose(b[shift:], a[:-shift], rtol=0, atol=1e-9 * np.abs(a).max())
    assert not b[:shift].any()


def test_zero_source_gives_zero_traces():
    inp = load_case_inputs("3d_small")
    inp.icmat = np.zeros_like(inp.icmat)
    assert not run_oracle(inp, 30).any()


def test_air_cells_record_zero():
    inp = load_case_inputs("2d_air_beta")
    o = Oracle(inp)
    o.run(60)
    assert np.all(o.state.p.reshape(-1)[o.icczero] == 0.0)


def test_hard_source_sets_pressure():
    inp = load_case_inputs("2d_small")
    inp.outc = inp.icc[:4].copy()
    out = run_oracle(inp, 50)
    np.testing.assert_allclose(out, inp.icmat[:4, :50].T.astype(np.float64), rtol=0, atol=0)


def test_wavefront_speed_in_homogeneous_lossless_medium():
    """A plane wave from the source rows reaches a row L cells away after ~L/(c dt/dx) steps."""
    inp = load_case_inputs("2d_nopml")
    for k in ("apmlu1", "apmlu2", "apmlx1", "apmlx2"):
        inp.maps[k] = np.zeros_like(inp.maps[k])
    for k in ("bpmlu1", "bpmlu2", "bpmlx1", "bpmlx2", "kappax", "kappau"):
        inp.maps[k] = np.ones_like(inp.maps[k])
    c0 = 1540.0
    inp.maps["c"] = np.full_like(inp.maps["c"], c0)
    inp.maps["rho"] = np.full_like(inp.maps["rho"], 1000.0)
    inp.maps["K"] = np.full_like(inp.maps["K"], c0**2 * 1000.0)
    inp.dcmap = np.zeros_like(inp.dcmap)
    inp.dmap = inp.d[:, :, None].copy()
    # a single sensor column far from the source rows, every step
    row = 8 + 20
    inp.outc = np.array([[row, inp.shape[1] // 2]], dtype=np.int32)
    inp.mod_t = 1
    out = run_oracle(inp, inp.nt)[:, 0]
    cfl = c0 * inp.dt / inp.spacing[0]
    onset = np.argmax(np.abs(out) > 0.05 * np.abs(out).max())
    src = inp.icmat[0].astype(np.float64)
    src_onset = np.argmax(np.abs(src) > 0.05 * np.abs(src).max())
    expected = src_onset + (row - 8) / cfl
    assert abs(onset - expected) < 0.1 * (row - 8) / cfl


@pytest.mark.parametrize("name", ["2d_aniso", "3d_aniso"])
def test_anisotropic_maps_equal_across_directions_give_isotropic_result(name):
    """The reference's own pre-processing gives every direction the same maps
    (pml_builder.py:926-1025 ramps all of them alike), so dropping the extra maps is exact."""
    from fullwave25_gb300.inputs import anisotropic_extra_maps

    inp = load_case_inputs(name)
    assert not inp.isotropic
    iso = load_case_inputs(name)
    iso.maps = {k: v for k, v in iso.maps.items() if k not in anisotropic_extra_maps(iso.ndim)}
    assert iso.isotropic
    np.testing.assert_array_equal(run_oracle(inp, 40), run_oracle(iso, 40))


def test_truly_anisotropic_maps_change_the_result():
    inp = load_case_inputs("2d_aniso")
    base = run_oracle(inp, 80)
    inp.maps = dict(inp.maps)
    inp.maps["apmlw1"] = (inp.maps["apmlw1"] * np.float32(3.0)).astype(np.float32)
    assert rel_l2(run_oracle(inp, 80), base) > 1e-6
