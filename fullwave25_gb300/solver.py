"""In-memory solver with the reference ``Solver`` interface (fullwave/solver/solver.py:276-778).

``Solver(work_dir, grid, medium, source, sensor, ...).run()`` builds the PML-extended maps with
this package's host builders (the reference's PMLBuilder/InputFileWriter arithmetic, no files),
runs the GB300 engine and returns the traces reshaped exactly as ``Solver._reshape_sensor_data``
does: ``raw.reshape(-1, n_sensors).T`` -> ``[n_sensors, n_out]`` (solver.py:599-618).
"""

from __future__ import annotations

import logging
import time
from pathlib import Path

import numpy as np

from .exponential import PMLBuilderExponentialAttenuation
from .inputs import build_inputs, build_inputs_exponential, write_simulation_dir
from .medium import Medium
from .pml import PMLBuilder
from .source import Sensor

logger = logging.getLogger("__main__." + __name__)


class Solver:
    def __init__(self, work_dir: Path, grid, medium, source=None, sensor=None, *,
                 transducer=None, path_fullwave_simulation_bin: Path | None = None,
                 use_pml: bool = True, m_spatial_order: int = 8,
                 pml_layer_thickness_px: int | None = None, n_transition_layer: int | None = None,
                 run_on_memory: bool = False, use_gpu: bool = True,
                 use_exponential_attenuation: bool = False, use_isotropic_relaxation: bool = True,
                 cuda_device_id: str | int | list | None = None) -> None:
        if not use_gpu:
            raise NotImplementedError("Currently, only GPU version is supported.")
        if transducer is not None:
            if source is not None or sensor is not None:
                raise ValueError("transducer must not be given together with source or sensor")
            source, sensor = transducer.source, transducer.sensor
        if source is None:
            raise ValueError("source or transducer must be provided")
        if sensor is None:
            raise ValueError("sensor or transducer must be provided")
        source.validate(grid.shape)
        sensor.validate(grid.shape)
        self.work_dir = Path(work_dir)
        self.grid, self.medium, self.source, self.sensor = grid, medium, source, sensor
        self.is_3d = grid.is_3d
        self.use_pml = use_pml
        if not use_pml:
            pml_layer_thickness_px = 0
            n_transition_layer = 0
        if pml_layer_thickness_px is None:
            pml_layer_thickness_px = grid.ppw * 3
        if n_transition_layer is None:
            n_transition_layer = grid.ppw * 3
        self.cuda_device_id = cuda_device_id
        self.use_isotropic_relaxation = use_isotropic_relaxation
        self.use_exponential_attenuation = use_exponential_attenuation
        medium.use_isotropic_relaxation = use_isotropic_relaxation   # as solver.py:457-476 does
        if use_exponential_attenuation:
            if not isinstance(medium, Medium):
                raise TypeError("the exponential-attenuation engine needs a Medium (alpha_coeff)")
            self.pml_builder = PMLBuilderExponentialAttenuation(
                grid, medium.sound_speed, medium.density, medium.alpha_coeff, medium.beta,
                source, sensor, air_map=medium.air_map, m_spatial_order=m_spatial_order,
                n_pml_layer=pml_layer_thickness_px)
        else:
            maps = medium.build() if isinstance(medium, Medium) else medium
            self.pml_builder = PMLBuilder(grid, maps, source, sensor,
                                          m_spatial_order=m_spatial_order,
                                          n_pml_layer=pml_layer_thickness_px,
                                          n_transition_layer=n_transition_layer,
                                          use_isotropic_relaxation=use_isotropic_relaxation)
        self.last_timing: dict = {}

    @staticmethod
    def _reshape_sensor_data(raw_sensor_output: np.ndarray, sensor) -> np.ndarray:
        return raw_sensor_output.reshape(-1, sensor.n_sensors).T

    def build_engine_inputs(self, *, record_whole_domain: bool = False,
                            sampling_modulus_time_whole_domain: int = 1):
        ext_medium = self.pml_builder.run(use_pml=self.use_pml)
        if self.use_exponential_attenuation:
            sensor = (Sensor(np.ones(self.pml_builder.extended_grid.shape, dtype=bool),
                             sampling_modulus_time=sampling_modulus_time_whole_domain)
                      if record_whole_domain else self.pml_builder.extended_sensor)
            return build_inputs_exponential(self.pml_builder.extended_grid, ext_medium,
                                            self.pml_builder.extended_source, sensor), sensor
        if not self.use_isotropic_relaxation and not self.use_pml:
            ext_medium.relaxation_param_dict_for_fw2 = ext_medium.calc_relaxation_param_dict_for_fw2(
                use_isotropic_relaxation=False)
        if record_whole_domain:
            sensor = Sensor(np.ones(self.pml_builder.extended_grid.shape, dtype=bool),
                            sampling_modulus_time=sampling_modulus_time_whole_domain)
        else:
            sensor = self.pml_builder.extended_sensor
        inputs = build_inputs(self.pml_builder.extended_grid, ext_medium,
                              self.pml_builder.extended_source, sensor)
        return inputs, sensor

    def run(self, simulation_dir_name: str | Path = "txrx_0", *, is_static_map: bool = False,
            recalculate_pml: bool = True, record_whole_domain: bool = False,
            sampling_modulus_time_whole_domain: int = 1, load_results: bool = True):
        from .engine import Engine  # noqa: PLC0415
        from .launcher import _first_device  # noqa: PLC0415

        import torch  # noqa: PLC0415

        t0 = time.time()
        inputs, sensor = self.build_engine_inputs(
            record_whole_domain=record_whole_domain,
            sampling_modulus_time_whole_domain=sampling_modulus_time_whole_domain)
        t1 = time.time()
        with torch.cuda.device(_first_device(self.cuda_device_id)):
            with Engine(inputs) as eng:
                raw = eng.run()
        t2 = time.time()
        self.last_timing = {"preprocess_s": t1 - t0, "engine_s": t2 - t1}
        if not load_results:
            sim_dir = self.work_dir / simulation_dir_name
            write_simulation_dir(inputs, sim_dir)
            raw.tofile(sim_dir / "genout.dat")
            return sim_dir / "genout.dat"
        return self._reshape_sensor_data(raw.reshape(-1), sensor)
