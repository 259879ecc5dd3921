"""Source signal: the Gaussian-modulated sinusoid of ``fullwave/utils/pulse.py:7-72``.

The expression and its floating-point operation order follow the reference, so the same
arguments give the same float64 samples (checked against reference-generated signals).
"""

from __future__ import annotations

import numpy as np


def gaussian_modulated_sinusoidal_signal(nt: int, duration: float, ncycles: int, drop_off: int,
                                         f0: float, p0: float, delay_sec: float = 0.0,
                                         i_layer: int | None = None,
                                         dt_for_layer_delay: float | None = None,
                                         cfl_for_layer_delay: float | None = None) -> np.ndarray:
    """``p0 * exp(-(1.05 t w0 / (ncycles pi))^(2 drop_off)) * sin(w0 t)`` on ``nt`` samples.

    The sample times span ``duration`` and start at ``-ncycles / f0``; ``delay_sec`` delays the
    pulse, and a source layer ``i_layer`` cells deep adds ``i_layer * dt / cfl`` (one cell of
    travel at the reference speed per layer), for which both ``dt_for_layer_delay`` and
    ``cfl_for_layer_delay`` are required (AssertionError otherwise, as in the reference).
    """
    omega0 = 2 * np.pi * f0
    t = np.arange(0, nt) / nt * duration - ncycles / f0
    t = t - delay_sec
    if i_layer:
        assert dt_for_layer_delay, "a layer delay (i_layer) needs dt_for_layer_delay"
        assert cfl_for_layer_delay, "a layer delay (i_layer) needs cfl_for_layer_delay"
        t = t - (dt_for_layer_delay / cfl_for_layer_delay) * i_layer
    envelope = np.exp(-((1.05 * t * omega0 / (ncycles * np.pi)) ** (2 * drop_off)))
    return envelope * np.sin(t * omega0) * p0
