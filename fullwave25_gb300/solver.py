"""In-memory solver with the reference ``Solver`` interface (fullwave/solver/solver.py:276-778).

``Solver(work_dir, grid, medium, source, sensor, ...).run()`` builds the PML-extended engine
inputs, runs the GB300 engine and returns the traces reshaped exactly as
``Solver._reshape_sensor_data`` does: ``raw.reshape(-1, n_sensors).T`` -> ``[n_sensors, n_out]``
(solver.py:599-618).

Pre-processing runs on the GPU by default (``device_build.device_inputs``: padding, relaxation
table lookup, mechanism sort, PML ramps, recursive-convolution coefficients, K and the tap-index
map, in float64 with the host builders' arithmetic); ``preprocess_on_device=False`` uses this
package's host builders (``pml.PMLBuilder`` and ``inputs.build_inputs``, the reference's
arithmetic in NumPy), which give the same maps.

Transmit sequences on one medium (``run(is_static_map=True, recalculate_pml=...)``): the
reference writes the medium's ``.dat`` maps into the work directory once and, for later events
run with ``recalculate_pml=False``, rewrites only ``icmat.dat`` and links the rest
(input_file_writer.py:145-169, :647-714). Here the medium stays resident on the GPU instead: a
static-map run keeps its engine (maps, tap table, coordinates) per work directory and device, and
a later ``recalculate_pml=False`` run of a solver on the same work directory only replaces the
source signals (``fw_set_source_signal``) and solves. As in the reference, such a run reuses the
first event's maps and source, sensor and air coordinates; here its source cells must be the
resident ones (``ValueError`` otherwise).
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

# Resident media of static-map transmit sequences: (work_dir, device) -> _Resident.
_RESIDENT: dict = {}


class _Resident:
    def __init__(self, engine, inputs, n_sensors, key_extra):
        self.engine, self.inputs, self.n_sensors, self.key_extra = engine, inputs, n_sensors, key_extra


def release_resident_media() -> None:
    """Free the device memory of every medium kept resident by static-map runs."""
    for r in _RESIDENT.values():
        r.engine.close()
    _RESIDENT.clear()


class Solver:
    def __init__(self, work_dir: Path, grid, medium, source=None, sensor=None, *,
                 transducer=None, path_fullwave_simulation_bin: Path | None = None,
                 use_pml: bool = True, m_spatial_order: int = 8,
                 pml_layer_thickness_px: int | None = None, n_transition_layer: int | None = None,
                 run_on_memory: bool = False, use_gpu: bool = True,
                 use_exponential_attenuation: bool = False, use_isotropic_relaxation: bool = True,
                 cuda_device_id: str | int | list | None = None,
                 preprocess_on_device: bool = True) -> None:
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
        self.pml_layer_thickness_px = int(pml_layer_thickness_px)
        self.n_transition_layer = int(n_transition_layer)
        self.m_spatial_order = m_spatial_order
        self.cuda_device_id = cuda_device_id
        self.use_isotropic_relaxation = use_isotropic_relaxation
        self.use_exponential_attenuation = use_exponential_attenuation
        self.preprocess_on_device = preprocess_on_device
        medium.use_isotropic_relaxation = use_isotropic_relaxation   # as solver.py:457-476 does
        if use_exponential_attenuation and not isinstance(medium, Medium):
            raise TypeError("the exponential-attenuation engine needs a Medium (alpha_coeff)")
        self._pml_builder = None
        self.last_timing: dict = {}

    @property
    def pml_builder(self):
        """The host PML builder (built on first use; the device path does not need it)."""
        if self._pml_builder is None:
            m = self.medium
            if self.use_exponential_attenuation:
                self._pml_builder = PMLBuilderExponentialAttenuation(
                    self.grid, m.sound_speed, m.density, m.alpha_coeff, m.beta, self.source,
                    self.sensor, air_map=m.air_map, m_spatial_order=self.m_spatial_order,
                    n_pml_layer=self.pml_layer_thickness_px)
            else:
                maps = m.build() if isinstance(m, Medium) else m
                self._pml_builder = PMLBuilder(
                    self.grid, maps, self.source, self.sensor,
                    m_spatial_order=self.m_spatial_order,
                    n_pml_layer=self.pml_layer_thickness_px,
                    n_transition_layer=self.n_transition_layer,
                    use_isotropic_relaxation=self.use_isotropic_relaxation)
        return self._pml_builder

    @staticmethod
    def _reshape_sensor_data(raw_sensor_output: np.ndarray, sensor) -> np.ndarray:
        n = sensor if isinstance(sensor, (int, np.integer)) else sensor.n_sensors
        return raw_sensor_output.reshape(-1, n).T

    def build_engine_inputs(self, *, record_whole_domain: bool = False,
                            sampling_modulus_time_whole_domain: int = 1):
        """Host-built engine inputs (NumPy) and the extended sensor."""
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

    def build_device_inputs(self, *, record_whole_domain: bool = False,
                            sampling_modulus_time_whole_domain: int = 1, device=None):
        """Engine inputs built on the GPU (``DeviceInputs``) and the number of sensors."""
        from .device_build import device_inputs  # noqa: PLC0415

        return device_inputs(
            self.grid, self.medium, self.source, self.sensor,
            n_pml=self.pml_layer_thickness_px, n_transition=self.n_transition_layer,
            use_pml=self.use_pml, use_isotropic_relaxation=self.use_isotropic_relaxation,
            use_exponential_attenuation=self.use_exponential_attenuation,
            m_spatial_order=self.m_spatial_order, record_whole_domain=record_whole_domain,
            sampling_modulus_time_whole_domain=sampling_modulus_time_whole_domain, device=device)

    def _resident_key(self, device_index: int):
        return (str(self.work_dir.resolve()), device_index)

    def run(self, simulation_dir_name: str | Path = "txrx_0", *, is_static_map: bool = False,
            recalculate_pml: bool = True, record_whole_domain: bool = False,
            sampling_modulus_time_whole_domain: int = 1, load_results: bool = True):
        from .engine import Engine  # noqa: PLC0415
        from .launcher import resolve_device  # noqa: PLC0415

        import torch  # noqa: PLC0415

        dev_index = resolve_device(self.cuda_device_id)
        key = self._resident_key(dev_index)
        key_extra = (record_whole_domain, sampling_modulus_time_whole_domain)
        resident = _RESIDENT.get(key) if is_static_map and not recalculate_pml else None
        if resident is not None and resident.key_extra != key_extra:
            resident = None
        t0 = time.perf_counter()
        timing = {"pml_rebuilt": resident is None, "maps_uploaded": resident is None,
                  "preprocess_on_device": self.preprocess_on_device}
        with torch.cuda.device(dev_index):
            if resident is not None:
                # later transmit event on the resident medium: only the source signals go up
                icc = resident.inputs.icc
                icc = icc.cpu().numpy() if hasattr(icc, "cpu") else np.asarray(icc)
                nb = (resident.inputs.shape[0] - self.grid.shape[0]) // 2
                if (tuple(n + 2 * nb for n in self.grid.shape) != tuple(resident.inputs.shape)
                        or self.grid.nt != resident.inputs.nt):
                    raise ValueError("a static-map run with recalculate_pml=False must use the "
                                     "grid (shape and nt) of the resident medium")
                if (self.source.incoords.shape != icc.shape
                        or not np.array_equal(self.source.incoords + nb, icc)):
                    raise ValueError("a static-map run with recalculate_pml=False must drive the "
                                     "source cells of the resident medium")
                t1 = time.perf_counter()
                eng = resident.engine
                eng.set_source_signal(np.asarray(self.source.icmat, dtype=np.float32))
                t2 = time.perf_counter()
                raw = eng.run()
                t3 = time.perf_counter()
                n_sensors, inputs = resident.n_sensors, resident.inputs
                timing.update(preprocess_s=t1 - t0, upload_s=t2 - t1, engine_s=t3 - t2)
            else:
                if self.preprocess_on_device:
                    inputs, n_sensors = self.build_device_inputs(
                        record_whole_domain=record_whole_domain,
                        sampling_modulus_time_whole_domain=sampling_modulus_time_whole_domain)
                else:
                    inputs, sensor = self.build_engine_inputs(
                        record_whole_domain=record_whole_domain,
                        sampling_modulus_time_whole_domain=sampling_modulus_time_whole_domain)
                    n_sensors = sensor.n_sensors
                t1 = time.perf_counter()
                eng = Engine(inputs, validate=not self.preprocess_on_device)
                t2 = time.perf_counter()
                try:
                    raw = eng.run()
                except BaseException:
                    eng.close()
                    raise
                t3 = time.perf_counter()
                timing.update(preprocess_s=t1 - t0, upload_s=t2 - t1, engine_s=t3 - t2)
                if is_static_map:
                    old = _RESIDENT.pop(key, None)
                    if old is not None:
                        old.engine.close()
                    _RESIDENT[key] = _Resident(eng, inputs, n_sensors, key_extra)
                else:
                    eng.close()
        timing["total_s"] = time.perf_counter() - t0
        self.last_timing = timing
        if not load_results:
            sim_dir = self.work_dir / simulation_dir_name
            host = inputs if not hasattr(inputs, "make_engine") else _host_copy(inputs)
            write_simulation_dir(host, sim_dir)
            raw.tofile(sim_dir / "genout.dat")
            return sim_dir / "genout.dat"
        return self._reshape_sensor_data(raw.reshape(-1), n_sensors)


def _host_copy(dinp):
    from .workloads3d import to_host_inputs  # noqa: PLC0415

    return to_host_inputs(dinp)
