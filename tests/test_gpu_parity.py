"""GPU engine vs the FP64 oracle through the C ABI (``-m gpu``).

Tolerance: sensor traces of the FP32 engine within 1e-4 relative L2 of the FP64 oracle
(``||engine - oracle|| / ||oracle||``), the bar the benchmark configurations set.
Size-independent properties at the full plain-2D workload size (944 x 688 extended, 4000 steps):
bitwise determinism, bitwise time-shift invariance, linearity to 1e-5, finite output.
"""

import tempfile
from pathlib import Path

import numpy as np
import pytest

from fdtd_oracle import rel_l2, run_oracle
from golden_io import CASE_NAMES, HERE, load_case_inputs, write_case_dir

pytestmark = pytest.mark.gpu
TOL = 1e-4
TRACES = np.load(HERE / "oracle_traces.npz")


@pytest.mark.parametrize("name", CASE_NAMES)
def test_launcher_dropin_matches_oracle(engine_lib, cuda, name):
    from fullwave25_gb300 import Launcher

    with tempfile.TemporaryDirectory() as td:
        sim = write_case_dir(name, Path(td) / name)
        inp = load_case_inputs(name)
        launcher = Launcher(is_3d=inp.ndim == 3, cuda_device_id=0)
        flat = launcher.run(sim)
        assert flat.dtype == np.float32 and flat.ndim == 1
        assert (sim / "genout.dat").exists()
        got = flat.reshape(-1, inp.outc.shape[0])
        ref = TRACES[name]
        assert got.shape == ref.shape
        err = rel_l2(got, ref)
        assert err < TOL, f"{name}: rel-L2 {err:.3e}"
        assert launcher.run(sim, load_results=False) == sim / "genout.dat"


def test_launcher_reports_failure_as_simulation_error(engine_lib, cuda):
    from fullwave25_gb300 import Launcher, SimulationError

    with tempfile.TemporaryDirectory() as td:
        with pytest.raises(SimulationError):
            Launcher().run(Path(td))
        assert (Path(td) / "fw2_execution.log").exists()


def test_engine_rejects_out_of_grid_sensor_without_fault(engine_lib, cuda):
    from fullwave25_gb300.engine import Engine, EngineError

    inp = load_case_inputs("2d_small")
    inp.outc = inp.outc.copy()
    inp.outc[1, 1] = 10_000
    with pytest.raises(EngineError, match="FW_ERR_ARGUMENT"):
        Engine(inp, validate=False)
    # the context is still usable
    good = load_case_inputs("2d_small")
    with Engine(good) as eng:
        assert rel_l2(eng.run(), TRACES["2d_small"]) < TOL


def test_chunked_advance_equals_full_run(engine_lib, cuda):
    from fullwave25_gb300.engine import Engine

    inp = load_case_inputs("3d_small")
    with Engine(inp) as eng:
        full = eng.run()
        eng.reset()
        for n in (1, 64, 17, 38):
            eng.advance(n)
        assert eng.current_step == inp.nt
        chunked = eng.read_traces()
    np.testing.assert_array_equal(full, chunked)


def test_new_source_signal_reuses_medium(engine_lib, cuda):
    from fullwave25_gb300.engine import Engine

    inp = load_case_inputs("2d_small")
    with Engine(inp) as eng:
        eng.run()
        new = (np.roll(inp.icmat, 5, axis=1) * -0.5).astype(np.float32)
        eng.set_source_signal(new)
        got = eng.run()
    inp.icmat = new
    assert rel_l2(got, run_oracle(inp)) < TOL


def test_solver_api_small_problem(engine_lib, cuda):
    from fullwave25_gb300 import Solver
    from fullwave25_gb300.workloads import plain_2d_problem

    grid, medium, source, sensor, _ = plain_2d_problem(shape=(96, 80), nt=300, seed=3)
    solver = Solver(Path(tempfile.gettempdir()), grid, medium, source, sensor,
                    pml_layer_thickness_px=12, n_transition_layer=12)
    out = solver.run()
    assert out.shape == (sensor.n_sensors, 300)
    inputs, _ = solver.build_engine_inputs()
    ref = run_oracle(inputs).T
    assert rel_l2(out, ref) < TOL


def test_plain_2d_reduced_matches_oracle(engine_lib, cuda):
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads import plain_2d_inputs

    inp = plain_2d_inputs(shape=(192, 160), nt=500, n_pml=20, n_transition=20)
    with Engine(inp) as eng:
        got = eng.run()
    err = rel_l2(got, run_oracle(inp))
    assert err < TOL, f"rel-L2 {err:.3e}"


@pytest.fixture(scope="module")
def plain_2d_full():
    from fullwave25_gb300.workloads import plain_2d_inputs

    return plain_2d_inputs()


def test_full_size_determinism_linearity_shift(engine_lib, cuda, plain_2d_full):
    from fullwave25_gb300.engine import Engine

    inp = plain_2d_full
    with Engine(inp) as eng:
        a = eng.run()
        b = eng.run()
        np.testing.assert_array_equal(a, b)
        assert np.isfinite(a).all() and np.abs(a).max() > 0
        eng.set_source_signal((inp.icmat * np.float32(2.0)).astype(np.float32))
        c = eng.run()
        assert rel_l2(c, 2.0 * a) < 1e-5
        shift = 11
        sh = np.zeros_like(inp.icmat)
        sh[:, shift:] = inp.icmat[:, :-shift]
        eng.set_source_signal(sh)
        d = eng.run()
    np.testing.assert_array_equal(d[shift:], a[:-shift])
    assert not d[:shift].any()


from helpers import engine_with_variant as _engine_with_variant  # noqa: E402


@pytest.fixture(scope="module")
def plain_3d_small(cuda):
    from fullwave25_gb300.workloads3d import plain_3d_device_inputs, to_host_inputs

    d = plain_3d_device_inputs(shape=(48, 40, 72), nt=240, n_pml=8, n_transition=8,
                               sensor_plane=24, element_height=8)
    return d, to_host_inputs(d)


def test_march_kernels_equal_direct_kernels_bitwise(engine_lib, cuda, plain_3d_small):
    d, host = plain_3d_small
    with _engine_with_variant(host, "march") as em, _engine_with_variant(host, "direct") as ed:
        assert em.kernel_variant == "stream" and ed.kernel_variant == "direct"
        a, b = em.run(), ed.run()
    assert np.abs(a).max() > 0
    np.testing.assert_array_equal(a, b)


def test_plain_3d_reduced_matches_oracle(engine_lib, cuda, plain_3d_small):
    from fdtd_oracle_c import run_oracle_c

    d, host = plain_3d_small
    with d.make_engine() as eng:
        assert eng.kernel_variant == "stream"
        got = eng.run()
    err = rel_l2(got, run_oracle_c(host))
    assert err < TOL, f"rel-L2 {err:.3e}"


def test_device_and_host_inputs_give_same_traces(engine_lib, cuda, plain_3d_small):
    from fullwave25_gb300.engine import Engine

    d, host = plain_3d_small
    with d.make_engine() as a, Engine(host) as b:
        np.testing.assert_array_equal(a.run(), b.run())


def test_solver_whole_domain_recording_movie(engine_lib, cuda):
    """record_whole_domain=True records every cell of the extended grid every
    ``sampling_modulus_time_whole_domain`` steps; reshaped to [nt, nx, ny] each frame is the
    pressure field at that step (the last frame equals the field left in the engine)."""
    from fullwave25_gb300 import Solver
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.signal_process import reshape_whole_sensor_to_nt_nx_ny
    from fullwave25_gb300.workloads import plain_2d_problem

    nt, mod = 120, 4
    grid, medium, source, sensor, _ = plain_2d_problem(shape=(64, 48), nt=nt, seed=5)
    solver = Solver(Path(tempfile.gettempdir()), grid, medium, source, sensor,
                    pml_layer_thickness_px=8, n_transition_layer=8)
    out = solver.run(record_whole_domain=True, sampling_modulus_time_whole_domain=mod)
    ext = solver.pml_builder.extended_grid
    movie = reshape_whole_sensor_to_nt_nx_ny(out, ext)
    n_out = (nt + mod - 1) // mod
    assert movie.shape == (n_out, ext.nx, ext.ny)
    inputs, _ = solver.build_engine_inputs(record_whole_domain=True,
                                           sampling_modulus_time_whole_domain=mod)
    with Engine(inputs) as eng:
        eng.reset()
        eng.advance((n_out - 1) * mod + 1)   # the last recorded step is (n_out - 1) * mod
        np.testing.assert_array_equal(movie[-1], eng.get_field(0))
    assert np.abs(movie[-1]).max() > 0


def test_plain_3d_full_size_determinism_scaling_shift(engine_lib, cuda):
    """At the full plain 3D size (512^3 + PML = 656^3 cells), over the first 120 steps: bitwise
    determinism, linearity in the source (x2 within 1e-6 relative L2) and exact time-shift
    invariance (source delayed by 7 steps -> traces delayed by 7 steps, bitwise)."""
    from fullwave25_gb300.workloads3d import plain_3d_device_inputs

    d = plain_3d_device_inputs()
    n = 120
    icmat = d.icmat.cpu().numpy()
    with d.make_engine() as eng:
        def solve():
            eng.reset()
            eng.advance(n)
            return eng.read_traces(0, n)

        a = solve()
        np.testing.assert_array_equal(solve(), a)
        assert np.isfinite(a).all() and np.abs(a).max() > 0
        eng.set_source_signal((icmat * np.float32(2.0)).astype(np.float32))
        assert rel_l2(solve(), 2.0 * a) < 1e-6
        shift = 7
        sh = np.zeros_like(icmat)
        sh[:, shift:] = icmat[:, :-shift]
        eng.set_source_signal(sh)
        b = solve()
    np.testing.assert_array_equal(b[shift:], a[:-shift])
    assert not b[:shift].any()
