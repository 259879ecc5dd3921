"""Host restatements pinned to outputs of the reference's own code (CPU).

The fixtures were generated by importing the reference (``tests/golden/make_golden.py``):
* ``pulse.npz``: ``gaussian_modulated_sinusoidal_signal`` (fullwave/utils/pulse.py:7-72) for
  four parameter sets (cycle counts, drop-offs, delays, source-layer offsets); this package's
  ``pulse.py`` must give the same float64 samples exactly;
* ``transducer_post.npz``: ``Transducer.post_process_sensor_output`` (fullwave/transducer.py:
  807-869) of random per-sensor traces, for a linear and a convex array with inactive elements,
  with and without surface averaging; ``transducer.post_process_sensor_output`` must match, and
  so must the per-element weighted sums that ``fw_set_sensor_groups`` forms in the time loop
  (``element_groups``).
"""

import numpy as np
import pytest

from golden_io import HERE

PULSE = np.load(HERE / "pulse.npz")
TRANSDUCER = np.load(HERE / "transducer_post.npz")


@pytest.mark.parametrize("k", range(4))
def test_pulse_equals_reference(k):
    from fullwave25_gb300.pulse import gaussian_modulated_sinusoidal_signal

    nt, duration, ncyc, drop, f0, p0, delay, layer, dt, cfl = PULSE[f"params_{k}"]
    kw = dict(nt=int(nt), duration=duration, ncycles=int(ncyc), drop_off=int(drop), f0=f0, p0=p0,
              delay_sec=delay)
    if layer:
        kw.update(i_layer=int(layer), dt_for_layer_delay=dt, cfl_for_layer_delay=cfl)
    np.testing.assert_array_equal(gaussian_modulated_sinusoidal_signal(**kw), PULSE[f"signal_{k}"])


def test_pulse_layer_delay_needs_dt_and_cfl():
    from fullwave25_gb300.pulse import gaussian_modulated_sinusoidal_signal

    with pytest.raises(AssertionError):
        gaussian_modulated_sinusoidal_signal(100, 1e-6, 2, 2, 3e6, 1.0, i_layer=2)


def _layout(name):
    ids = TRANSDUCER[f"{name}/surface_id"]
    coords = TRANSDUCER[f"{name}/surface_coords"]
    n_el = TRANSDUCER[f"{name}/active"].shape[0]
    surfaces = {e: coords[ids == e].reshape(-1, 2) for e in range(1, n_el + 1)}
    return TRANSDUCER[f"{name}/outcoords"], surfaces, TRANSDUCER[f"{name}/active"]


@pytest.mark.parametrize("name", ["linear", "convex"])
@pytest.mark.parametrize("average", [True, False])
def test_post_processing_equals_reference(name, average):
    from fullwave25_gb300.transducer import element_groups, post_process_sensor_output

    outcoords, surfaces, active = _layout(name)
    traces = TRANSDUCER[f"{name}/traces"]
    ref = TRANSDUCER[f"{name}/{'averaged' if average else 'centre'}"]
    got = post_process_sensor_output(traces, outcoords, surfaces, active,
                                     average_surface_signals=average)
    assert got.dtype == ref.dtype and got.shape == ref.shape
    np.testing.assert_array_equal(got, ref)
    # the in-loop form: one group and one weight per sensor
    group, weight, n = element_groups(outcoords, surfaces, active, average_surface_signals=average)
    assert n == ref.shape[0]
    summed = np.zeros_like(ref)
    for k in range(outcoords.shape[0]):
        if group[k] >= 0:
            summed[group[k]] += weight[k] * traces[k]
    np.testing.assert_allclose(summed, ref, rtol=1e-6, atol=1e-6)
