"""GB300-native FDTD engine for Fullwave 2.5 simulations.

Public surface (names follow the reference package ``fullwave``):
``Grid``, ``MediumRelaxationMaps``, ``Source``, ``Sensor``, ``PMLBuilder``, ``Solver``,
``Launcher`` / ``SimulationError`` (drop-in for ``fullwave.solver.launcher``), ``signal_process``
(whole-domain output reshapes), and the engine binding ``Engine`` over the C ABI of
``include/fwgb.h``.
"""

import logging

from .grid import Grid
from .inputs import EngineInputs, build_inputs, load_dat_data, read_simulation_dir, write_simulation_dir
from .launcher import Launcher, SimulationError
from .exponential import MediumExponentialAttenuation, PMLBuilderExponentialAttenuation
from .medium import Medium, MediumRelaxationMaps
from .pml import PMLBuilder
from .pulse import gaussian_modulated_sinusoidal_signal
from . import signal_process
from .solver import Solver
from .source import Sensor, Source

__version__ = "0.1.0"

logging.getLogger("__main__." + __name__).addHandler(logging.NullHandler())

__all__ = [
    "EngineInputs", "Grid", "Launcher", "Medium", "MediumExponentialAttenuation",
    "MediumRelaxationMaps", "PMLBuilder", "PMLBuilderExponentialAttenuation", "Sensor",
    "SimulationError", "Solver", "Source", "build_inputs", "gaussian_modulated_sinusoidal_signal",
    "load_dat_data", "read_simulation_dir", "signal_process", "write_simulation_dir",
]
