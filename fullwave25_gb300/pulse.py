"""Source signal (mirrors ``fullwave/utils/pulse.py:7-72``)."""

from __future__ import annotations

import numpy as np


def gaussian_modulated_sinusoidal_signal(nt: int, duration: float, ncycles: int, drop_off: int,
                                         f0: float, p0: float, delay_sec: float = 0.0,
                                         i_layer: int | None = None,
                                         dt_for_layer_delay: float | None = None,
                                         cfl_for_layer_delay: float | None = None) -> np.ndarray:
    """``p0 * exp(-(1.05 t w0 / (ncycles pi))^(2 drop_off)) * sin(w0 t)`` on ``nt`` samples.

    ``t`` starts at ``-ncycles / f0`` and is further delayed by ``delay_sec`` and, for a source
    layer ``i_layer`` deep, by ``i_layer * dt / cfl`` (one cell of travel at ``c0``).
    """
    t = np.arange(0, nt) / nt * duration - ncycles / f0
    t = t - delay_sec
    if i_layer:
        assert dt_for_layer_delay, "dt must be provided if i_layer is provided"
        assert cfl_for_layer_delay, "cfl must be provided if i_layer is provided"
        t = t - (dt_for_layer_delay / cfl_for_layer_delay) * i_layer
    omega0 = 2 * np.pi * f0
    return np.multiply(np.exp(-((1.05 * t * omega0 / (ncycles * np.pi)) ** (2 * drop_off))),
                       np.sin(t * omega0)) * p0
