"""Drop-in replacement of ``fullwave.solver.launcher.Launcher`` backed by the GB300 engine.

The reference ``Launcher.run`` (fullwave/solver/launcher.py:160-254) changes into the simulation
directory, runs the closed engine executable, which reads the ``.dat`` input set and writes
``genout.dat``, and returns ``load_dat_data(genout.dat)``: a flat float32 array, time-major
``[n_out * ncoordsout]``. This class keeps that contract: same constructor arguments, same
``run(simulation_dir, load_results=...)`` signature and return values, same ``SimulationError``
on failure with the log in ``fw2_execution.log`` and ``NotImplementedError`` for CPU mode.
The time loop runs in-process on the GPU through the C ABI instead of in a subprocess.

Use it behind the reference API by replacing the solver's launcher::

    solver = fullwave.Solver(...)
    solver.fullwave_launcher = fullwave25_gb300.Launcher(is_3d=solver.is_3d)
    traces = solver.run()
"""

from __future__ import annotations

import logging
import time
from pathlib import Path

from .inputs import load_dat_data, read_simulation_dir

logger = logging.getLogger("__main__." + __name__)


class SimulationError(Exception):
    """Exception raised for errors in the simulation."""


def device_list(cuda_device_id) -> list:
    """The device ids named by ``cuda_device_id`` (None, an int, "0,1,2" or a list), as the
    reference reads them to set CUDA_VISIBLE_DEVICES (launcher.py:64-105, :206)."""
    if cuda_device_id is None:
        return [0]
    if isinstance(cuda_device_id, (list, tuple)):
        if not cuda_device_id:
            raise ValueError("cuda_device_id list is empty")
        return [int(v) for v in cuda_device_id]
    ids = [v.strip() for v in str(cuda_device_id).split(",") if v.strip()]
    if not ids:
        raise ValueError(f"cuda_device_id {cuda_device_id!r} names no device")
    return [int(v) for v in ids]


_WARNED_MULTI: set = set()


def resolve_device(cuda_device_id) -> int:
    """The device one simulation runs on: the first listed id. The reference splits one
    simulation into depth slabs across every listed GPU inside its executables; this engine runs
    a simulation on one GPU (depth slabs exist as a tested decomposition, ``slabs.py``, without a
    peer-to-peer transport), so when several ids are listed it says so once and uses the first."""
    ids = device_list(cuda_device_id)
    if len(ids) > 1 and tuple(ids) not in _WARNED_MULTI:
        _WARNED_MULTI.add(tuple(ids))
        logger.warning("cuda_device_id lists %d GPUs %s: one simulation runs on one GPU here; "
                       "using GPU %d (run independent simulations on the others)", len(ids), ids,
                       ids[0])
    return ids[0]


_first_device = resolve_device


class Launcher:
    """Runs one simulation directory on one GPU (the engine is single-GPU)."""

    def __init__(self, path_fullwave_simulation_bin: Path | None = None, *, is_3d: bool = False,
                 use_gpu: bool = True, cuda_device_id: str | int | list | None = None) -> None:
        # The executable path is accepted for signature compatibility; nothing is executed.
        self._path_fullwave_simulation_bin = path_fullwave_simulation_bin
        self.is_3d = is_3d
        self.use_gpu = use_gpu
        self.device_ids = device_list(cuda_device_id)
        self.device_index = resolve_device(cuda_device_id)
        self.cuda_device_id = ",".join(str(v) for v in self.device_ids)
        self.last_timing: dict = {}

    def run(self, simulation_dir: Path, *, load_results: bool = True):
        """Run the simulation in ``simulation_dir``; returns the flat genout array or its path."""
        from .engine import Engine  # noqa: PLC0415  (loads the native library)

        simulation_dir = Path(simulation_dir).absolute()
        if not self.use_gpu:
            message = "Currently, only GPU version is supported."
            logger.error(message)
            raise NotImplementedError(message)
        log_path = simulation_dir / "fw2_execution.log"
        genout = simulation_dir / "genout.dat"
        t0 = time.time()
        try:
            import torch  # noqa: PLC0415

            inputs = read_simulation_dir(simulation_dir)
            if inputs.ndim != (3 if self.is_3d else 2):
                raise ValueError(f"simulation directory is {inputs.ndim}D, launcher is_3d={self.is_3d}")
            with torch.cuda.device(self.device_index):
                with Engine(inputs) as eng:
                    t1 = time.time()
                    traces = eng.run()
                    t2 = time.time()
            traces.tofile(genout)
            self.last_timing = {"read_s": t1 - t0, "run_s": t2 - t1, "total_s": time.time() - t0}
            log_path.write_text(
                f"fullwave25_gb300 engine: grid {inputs.shape}, nT {inputs.nt}, "
                f"{inputs.icc.shape[0]} sources, {inputs.outc.shape[0]} sensors\n"
                f"Simulation completed in {t2 - t1:.3e} seconds.\n", encoding="utf-8")
            logger.info("Simulation completed in %.2e seconds.", t2 - t1)
        except Exception as e:
            log_path.write_text(f"fullwave25_gb300 engine failed: {e!r}\n", encoding="utf-8")
            logger.exception("Simulation failed")
            raise SimulationError(
                "Simulation failed. please check the simulation log file for more information.\n"
                f"The log file is located at:\n{log_path}") from e
        if load_results:
            return load_dat_data(genout)
        return genout
