"""Element grouping of sensor traces (host side)."""

import numpy as np
import pytest

from fullwave25_gb300.transducer import element_groups, post_process_sensor_output


def _layout(n_elements=6, width=4, row=5):
    outcoords = np.array([[row, j] for j in range(n_elements * width)])
    surfaces = {e + 1: np.array([[row, j] for j in range(e * width, (e + 1) * width)])
                for e in range(n_elements)}
    active = np.ones(n_elements, dtype=bool)
    active[2] = False
    return outcoords, surfaces, active


@pytest.mark.parametrize("average", [True, False])
def test_groups_reproduce_post_processing(average):
    outcoords, surfaces, active = _layout()
    rng = np.random.default_rng(0)
    traces = rng.standard_normal((outcoords.shape[0], 50)).astype(np.float32)
    ref = post_process_sensor_output(traces, outcoords, surfaces, active,
                                     average_surface_signals=average)
    g, w, n = element_groups(outcoords, surfaces, active, average_surface_signals=average)
    assert n == active.sum() == ref.shape[0]
    got = np.zeros_like(ref)
    for k in range(outcoords.shape[0]):
        if g[k] >= 0:
            got[g[k]] += w[k] * traces[k]
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6)
    assert (g == -1).sum() == (4 if average else outcoords.shape[0] - n)


def test_sensor_on_two_elements_is_rejected():
    outcoords, surfaces, active = _layout()
    surfaces[2] = np.vstack([surfaces[2], surfaces[1][:1]])
    with pytest.raises(ValueError, match="two elements"):
        element_groups(outcoords, surfaces, active)
