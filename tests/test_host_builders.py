"""Host pre-processing (grid, relaxation coefficients, PML, coordinates, file contract) against
the reference's own .dat output for the golden cases: byte-for-byte equality."""

import tempfile
from pathlib import Path

import numpy as np
import pytest

from fullwave25_gb300.inputs import read_simulation_dir, write_simulation_dir
from golden_io import CASE_NAMES, load_case, load_case_inputs, rebuild_case_inputs

INT_FILES = {"dcmap", "icc", "outc", "icczero", "nX", "nY", "nZ", "nT", "nTic", "modT",
             "ncoords", "ncoordsout", "ncoordszero", "ndmap"}


@pytest.mark.parametrize("name", CASE_NAMES)
def test_rebuilt_dat_files_equal_reference(name):
    z = load_case(name)
    inp = rebuild_case_inputs(name)
    with tempfile.TemporaryDirectory() as td:
        write_simulation_dir(inp, Path(td))
        ref_files = {k[4:] for k in z.files if k.startswith("dat/")}
        mine = {p.stem for p in Path(td).glob("*.dat")}
        assert ref_files == mine
        for stem in sorted(ref_files):
            ref = z[f"dat/{stem}"].tobytes()
            got = (Path(td) / f"{stem}.dat").read_bytes()
            if ref != got:
                dt = np.int32 if stem in INT_FILES else np.float32
                a, b = np.frombuffer(ref, dt), np.frombuffer(got, dt)
                pytest.fail(f"{stem}.dat differs: sizes {a.size}/{b.size}, "
                            f"max diff {np.max(np.abs(a.astype(float) - b)) if a.size == b.size else 'n/a'}")


@pytest.mark.parametrize("name", CASE_NAMES)
def test_read_write_roundtrip(name):
    inp = load_case_inputs(name)
    with tempfile.TemporaryDirectory() as td:
        write_simulation_dir(inp, Path(td))
        back = read_simulation_dir(Path(td))
    assert back.shape == inp.shape and back.nt == inp.nt and back.mod_t == inp.mod_t
    for k in inp.maps:
        np.testing.assert_array_equal(back.maps[k], inp.maps[k])
    for k in ("icc", "outc", "icczero", "icmat", "dcmap", "dmap", "d"):
        np.testing.assert_array_equal(getattr(back, k), getattr(inp, k))


def test_missing_file_raises():
    with tempfile.TemporaryDirectory() as td:
        with pytest.raises(ValueError, match="does not exist"):
            read_simulation_dir(Path(td))


def test_validate_rejects_bad_coordinates():
    inp = load_case_inputs("2d_small")
    inp.outc = inp.outc.copy()
    inp.outc[0, 0] = inp.shape[0]
    with pytest.raises(ValueError, match="outside the grid"):
        inp.validate()


def test_grid_arithmetic_matches_reference_formulas():
    from fullwave25_gb300 import Grid

    g = Grid(domain_size=(3e-2, 2e-2), f0=3e6, duration=3e-2 / 1540 * 2, c0=1540)
    assert g.dx == pytest.approx(1540 / 3e6 / 12)
    assert g.dt == pytest.approx(0.2 * g.dx / 1540)
    assert g.shape == (int(np.round(3e-2 / g.dx)), int(np.round(2e-2 / g.dx)))
    assert g.nt == round(g.duration / g.dt)
    with pytest.raises(AssertionError):
        Grid(domain_size=(1e-2, 1e-2), f0=3e6, duration=1e-6, cfl=0.6)


def test_coordinate_order_is_row_major():
    from fullwave25_gb300 import Sensor, Source

    mask = np.zeros((4, 5), dtype=bool)
    mask[[0, 0, 2, 3], [4, 1, 2, 0]] = True
    s = Sensor(mask)
    np.testing.assert_array_equal(s.outcoords, [[0, 1], [0, 4], [2, 2], [3, 0]])
    with pytest.raises(ValueError):
        Source(np.zeros((3, 10)), mask)


def test_relaxation_coefficients_formula():
    """a/b as in the reference's known-answer test (tests/test_medium.py:645-654)."""
    from fullwave25_gb300.medium import calc_a_and_b

    d, k, al, dt = 2.0e4, 1.002, 1.5e7, 5e-9
    a, b = calc_a_and_b(d, k, al, dt)
    eb = np.exp(-(d / k + al) * dt)
    np.testing.assert_allclose(b, eb, rtol=1e-12)
    np.testing.assert_allclose(a, d / (k * (d + k * al) + 1e-10) * (eb - 1), rtol=1e-12)


def test_plain_2d_workload_physics_variants():
    """The plain 2D workload through the anisotropic-relaxation builder (every direction's map set
    equals the isotropic set, the reference builder's structure) and through the
    exponential-attenuation builder (PML 40 + 8 ghost cells, a_exp in [0, 1))."""
    from fullwave25_gb300.inputs import anisotropic_extra_maps
    from fullwave25_gb300.workloads import algorithmic_bytes_per_cell, plain_2d_inputs

    iso = plain_2d_inputs()
    an = plain_2d_inputs(physics="aniso")
    an.validate()
    assert not an.isotropic and set(an.maps) == set(iso.maps) | set(anisotropic_extra_maps(2))
    for k in iso.maps:
        np.testing.assert_array_equal(an.maps[k], iso.maps[k])
    np.testing.assert_array_equal(an.maps["apmly1"], iso.maps["apmlx1"])
    ex = plain_2d_inputs(physics="exp")
    ex.validate()
    assert ex.exponential and ex.shape == (864, 608)
    assert 0 <= ex.maps["a_exp"].min() and ex.maps["a_exp"].max() < 1
    np.testing.assert_array_equal(ex.icmat, iso.icmat)
    assert [algorithmic_bytes_per_cell(2, physics=p) for p in ("isotropic", "aniso", "exp")] == \
        [136, 176, 40]
    assert [algorithmic_bytes_per_cell(3, physics=p) for p in ("isotropic", "aniso", "exp")] == \
        [176, 256, 48]
