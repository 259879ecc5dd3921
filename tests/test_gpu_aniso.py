"""Anisotropic relaxation engine (one set of relaxation maps per derivative axis) on the GPU."""

import numpy as np
import pytest

from fdtd_oracle import rel_l2
from golden_io import load_case_inputs

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _skew(inp):
    """Make the maps really direction-dependent (the reference's builder gives equal ones)."""
    inp.maps = dict(inp.maps)
    for name, f in (("apmlw1", 3.0), ("bpmlw2", 0.97), ("kappay", 1.01), ("apmly2", 0.5),
                    ("apmlv1", 2.0), ("kappaz", 0.995)):
        if name in inp.maps:
            inp.maps[name] = (inp.maps[name] * np.float32(f)).astype(np.float32)
    return inp


@pytest.mark.parametrize("name", ["2d_aniso", "3d_aniso"])
def test_direction_dependent_maps_match_oracle(engine_lib, cuda, name):
    from fdtd_oracle_c import run_oracle_c
    from fullwave25_gb300.engine import Engine

    inp = _skew(load_case_inputs(name))
    with Engine(inp) as eng:
        got = eng.run()
    err = rel_l2(got, run_oracle_c(inp))
    assert err < TOL, f"{name}: rel-L2 {err:.3e}"


def test_aniso_march_equals_direct_bitwise(engine_lib, cuda):
    from helpers import engine_with_variant as _engine_with_variant

    inp = _skew(load_case_inputs("3d_aniso"))
    with _engine_with_variant(inp, "march") as a, _engine_with_variant(inp, "direct") as b:
        assert a.kernel_variant == "march" and b.kernel_variant == "direct"
        np.testing.assert_array_equal(a.run(), b.run())


def test_solver_anisotropic_equals_isotropic_for_equal_maps(engine_lib, cuda, tmp_path):
    from fullwave25_gb300 import Solver
    from fullwave25_gb300.workloads import plain_2d_problem

    outs = []
    for iso in (True, False):
        grid, medium, source, sensor, _ = plain_2d_problem(shape=(80, 72), nt=240, seed=4)
        s = Solver(tmp_path, grid, medium, source, sensor, pml_layer_thickness_px=10,
                   n_transition_layer=10, use_isotropic_relaxation=iso)
        inputs, _ = s.build_engine_inputs()
        assert inputs.isotropic == iso
        outs.append(s.run())
    np.testing.assert_array_equal(outs[0], outs[1])
