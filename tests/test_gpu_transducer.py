"""Per-element traces recorded inside the time loop equal the host post-processing of the
per-sensor traces."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("average", [True, False])
def test_in_loop_element_traces(engine_lib, cuda, average):
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.transducer import element_groups, post_process_sensor_output
    from fullwave25_gb300.workloads import plain_2d_inputs

    inp = plain_2d_inputs(shape=(96, 64), nt=300, n_pml=10, n_transition=10)
    width = 4
    outcoords = inp.outc
    n_el = outcoords.shape[0] // width
    surfaces = {e + 1: outcoords[e * width:(e + 1) * width] for e in range(n_el)}
    active = np.ones(n_el, dtype=bool)
    active[::5] = False
    with Engine(inp) as eng:
        per_sensor = eng.run()
        ref = post_process_sensor_output(per_sensor.T, outcoords, surfaces, active,
                                         average_surface_signals=average)
        g, w, n = element_groups(outcoords, surfaces, active, average_surface_signals=average)
        eng.set_sensor_groups(g, w, n)
        got = eng.run()
        assert got.shape == (inp.n_out, n)
        eng.set_sensor_groups(g, w, 0)
        np.testing.assert_array_equal(eng.run(), per_sensor)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(got.T, ref, rtol=0, atol=2e-6 * scale)
