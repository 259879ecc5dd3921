"""The reference ``Solver`` API on the GPU (``-m gpu``): pre-processing on the device, and transmit
sequences on a resident medium (``run(is_static_map=True, recalculate_pml=False)``,
fullwave/solver/solver.py:620-668, input_file_writer.py:145-169)."""

import tempfile
from pathlib import Path

import numpy as np
import pytest

from fdtd_oracle import rel_l2
from fdtd_oracle_c import run_oracle_c

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _problem(seed=3, shape=(96, 80), nt=300):
    from fullwave25_gb300.workloads import plain_2d_problem

    return plain_2d_problem(shape=shape, nt=nt, seed=seed)


def _ulp_diff(a, b):
    a = np.ascontiguousarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.ascontiguousarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


@pytest.mark.parametrize("iso", [True, False])
def test_device_preprocessing_gives_host_preprocessing_traces(engine_lib, cuda, iso):
    """Maps built on the GPU equal the host builders' (float64 exp/log on the GPU may differ from
    NumPy's by an ulp before the float32 rounding: at most 1 float32 ulp in 1e-4 of the entries is
    allowed); the traces are then equal, or within 1e-6 where a map entry differed."""
    from fullwave25_gb300 import Solver
    from fullwave25_gb300.workloads3d import to_host_inputs

    grid, medium, source, sensor, _ = _problem()
    out = {}
    for on_device in (True, False):
        s = Solver(Path(tempfile.gettempdir()), grid, medium, source, sensor,
                   pml_layer_thickness_px=12, n_transition_layer=12,
                   use_isotropic_relaxation=iso, preprocess_on_device=on_device)
        out[on_device] = s.run()
        assert s.last_timing["preprocess_on_device"] == on_device
    host, _ = s.build_engine_inputs()
    dev = to_host_inputs(s.build_device_inputs()[0])
    n_diff = 0
    for k in host.maps:
        u = _ulp_diff(dev.maps[k], host.maps[k])
        assert u.max() <= 1, k
        n_diff += int((u > 0).sum())
    np.testing.assert_array_equal(dev.dcmap, host.dcmap)
    assert n_diff <= 1e-4 * host.n_cells * len(host.maps)
    if n_diff == 0:
        np.testing.assert_array_equal(out[True], out[False])
    else:
        assert rel_l2(out[True], out[False]) < 1e-6
    assert rel_l2(out[True], run_oracle_c(host).T) < TOL


def _problem_3d(shape=(26, 24, 22), nt=150, physics="isotropic", seed=5):
    from fullwave25_gb300.grid import Grid
    from fullwave25_gb300.medium import Medium, MediumRelaxationMaps
    from fullwave25_gb300.pulse import gaussian_modulated_sinusoidal_signal
    from fullwave25_gb300.relaxation import default_table
    from fullwave25_gb300.source import Sensor, Source

    rng = np.random.default_rng(seed)
    grid = Grid.from_cells(shape, f0=3e6, nt=nt, ppw=12, cfl=0.2)
    c = 1540 + 40 * rng.standard_normal(shape).clip(-2, 2)
    rho = 1000 + 50 * rng.standard_normal(shape).clip(-2, 2)
    a0 = rng.uniform(0.3, 1.0, shape)
    gam = np.full(shape, 1.1)
    if physics == "exp":
        medium = Medium(grid, c, rho, a0, gam, np.zeros(shape))
    else:
        medium = MediumRelaxationMaps(grid, c, rho, np.zeros(shape),
                                      default_table().lookup(a0, gam))
    mask = np.zeros(shape, dtype=bool)
    mask[0, 4:-4, 4:-4] = True
    sig = gaussian_modulated_sinusoidal_signal(nt=nt, duration=grid.duration, ncycles=2,
                                               drop_off=2, f0=3e6, p0=1e5)
    smask = np.zeros(shape, dtype=bool)
    smask[6, ::3, ::3] = True
    return grid, medium, Source(np.tile(sig, (int(mask.sum()), 1)), mask), Sensor(smask)


@pytest.mark.parametrize("physics", ["isotropic", "aniso", "exp"])
def test_device_preprocessing_3d_gives_host_preprocessing_traces(engine_lib, cuda, physics):
    """The 3D engines through Solver.run(): GPU and NumPy pre-processing give the same maps (to
    the float32 ulp bound above) and traces, and the FP64 oracle's traces within 1e-4."""
    from fullwave25_gb300 import Solver
    from fullwave25_gb300.workloads3d import to_host_inputs

    grid, medium, source, sensor = _problem_3d(physics=physics)
    kw = dict(pml_layer_thickness_px=6, n_transition_layer=6,
              use_isotropic_relaxation=physics != "aniso",
              use_exponential_attenuation=physics == "exp")
    out = {}
    for on_device in (True, False):
        s = Solver(Path(tempfile.gettempdir()), grid, medium, source, sensor,
                   preprocess_on_device=on_device, **kw)
        out[on_device] = s.run()
    host, _ = s.build_engine_inputs()
    dev = to_host_inputs(s.build_device_inputs()[0])
    assert set(dev.maps) == set(host.maps)
    n_diff = 0
    for k in host.maps:
        u = _ulp_diff(dev.maps[k], host.maps[k])
        assert u.max() <= 1, k
        n_diff += int((u > 0).sum())
    assert n_diff <= 1e-4 * host.n_cells * len(host.maps)
    if n_diff == 0:
        np.testing.assert_array_equal(out[True], out[False])
    else:
        assert rel_l2(out[True], out[False]) < 1e-6
    assert np.abs(out[True]).max() > 0
    assert rel_l2(out[True], run_oracle_c(host).T) < TOL


def test_static_map_sequence_keeps_the_medium_resident(engine_lib, cuda):
    from fullwave25_gb300 import Solver
    from fullwave25_gb300.solver import release_resident_media
    from fullwave25_gb300.source import Source

    grid, medium, source, sensor, _ = _problem(seed=6)
    work = Path(tempfile.mkdtemp())
    # three transmit events on one medium: the source cells stay, the signals change
    signals = [source.p0, np.roll(source.p0, 7, axis=1) * -0.5,
               source.p0 * np.linspace(0.2, 1.0, source.p0.shape[0])[:, None]]
    try:
        got, timings = [], []
        for k, p0 in enumerate(signals):
            s = Solver(work, grid, medium, Source(p0, source.mask), sensor,
                       pml_layer_thickness_px=12, n_transition_layer=12)
            got.append(s.run(f"txrx_{k}", is_static_map=True, recalculate_pml=(k == 0)))
            timings.append(s.last_timing)
        assert timings[0]["pml_rebuilt"] and timings[0]["maps_uploaded"]
        for t in timings[1:]:
            assert not t["pml_rebuilt"] and not t["maps_uploaded"]
            assert t["preprocess_s"] < timings[0]["preprocess_s"]
        # each event equals a fresh solve of the same transmit
        for k, p0 in enumerate(signals):
            fresh = Solver(Path(tempfile.gettempdir()), grid, medium, Source(p0, source.mask),
                           sensor, pml_layer_thickness_px=12, n_transition_layer=12).run()
            np.testing.assert_array_equal(got[k], fresh, err_msg=f"transmit {k}")
        # a later event that drives other cells cannot reuse the resident medium
        mask = np.zeros_like(source.mask)
        mask[3, :10] = True
        other = Source(np.ones((10, grid.nt)), mask)
        s = Solver(work, grid, medium, other, sensor, pml_layer_thickness_px=12,
                   n_transition_layer=12)
        with pytest.raises(ValueError, match="source cells"):
            s.run("txrx_x", is_static_map=True, recalculate_pml=False)
        # nor one on another grid
        g2, m2, src2, sen2, _ = _problem(seed=6, nt=320)
        s = Solver(work, g2, m2, src2, sen2, pml_layer_thickness_px=12, n_transition_layer=12)
        with pytest.raises(ValueError, match="grid"):
            s.run("txrx_y", is_static_map=True, recalculate_pml=False)
    finally:
        release_resident_media()
