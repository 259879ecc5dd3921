"""Exponential-attenuation engine on the GPU (2D and 3D) against the FP64 oracle."""

import numpy as np
import pytest

from fdtd_oracle import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


@pytest.mark.parametrize("shape,nt", [((90, 70), 400), ((26, 24, 22), 150)])
def test_solver_exponential_matches_oracle(engine_lib, cuda, tmp_path, shape, nt):
    from fdtd_oracle_c import run_oracle_c
    from fullwave25_gb300 import Grid, Medium, Sensor, Solver, Source
    from fullwave25_gb300.pulse import gaussian_modulated_sinusoidal_signal

    rng = np.random.default_rng(7)
    grid = Grid.from_cells(shape, f0=3e6, nt=nt, ppw=12, cfl=0.2)
    c = 1540 + 40 * rng.standard_normal(shape).clip(-2, 2)
    medium = Medium(grid, c, np.full(shape, 1000.0), np.full(shape, 0.8), np.full(shape, 1.1),
                    np.zeros(shape))
    mask = np.zeros(shape, dtype=bool)
    mask[0] = True
    sig = gaussian_modulated_sinusoidal_signal(nt=nt, duration=grid.duration, ncycles=2,
                                               drop_off=2, f0=3e6, p0=1e5)
    source = Source(np.tile(sig, (int(mask.sum()), 1)), mask)
    smask = np.zeros(shape, dtype=bool)
    smask[6] = True
    sensor = Sensor(smask)
    solver = Solver(tmp_path, grid, medium, source, sensor, pml_layer_thickness_px=10,
                    use_exponential_attenuation=True)
    out = solver.run()
    inputs, _ = solver.build_engine_inputs()
    assert inputs.exponential
    ref = run_oracle_c(inputs).T
    assert np.abs(out).max() > 0
    assert rel_l2(out, ref) < TOL
