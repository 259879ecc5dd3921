"""Drop-in Launcher behaviour without a GPU, in the style of the reference's
tests/solver/test_launcher.py (the engine is replaced by a fake, as the reference replaces the
executable with a mocked subprocess)."""

import tempfile
from pathlib import Path

import numpy as np
import pytest

import fullwave25_gb300.engine as engine_mod
from fullwave25_gb300 import Launcher, SimulationError
from fullwave25_gb300.launcher import device_list, resolve_device
from golden_io import write_case_dir


class _FakeEngine:
    def __init__(self, inputs, **kw):
        self.inputs = inputs

    def run(self):
        return np.full((self.inputs.n_out, self.inputs.outc.shape[0]), 42.0, np.float32)

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


class _FailingEngine(_FakeEngine):
    def run(self):
        raise engine_mod.EngineError("fw_run", 2, "simulated CUDA failure")


class _FakeDevice:
    def __init__(self, idx):
        self.idx = idx

    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


@pytest.fixture
def sim_dir(tmp_path):
    return write_case_dir("2d_small", tmp_path / "txrx_0")


@pytest.fixture
def no_cuda(monkeypatch):
    import torch

    monkeypatch.setattr(torch.cuda, "device", _FakeDevice)


def test_run_success(sim_dir, monkeypatch, no_cuda):
    monkeypatch.setattr(engine_mod, "Engine", _FakeEngine)
    result = Launcher(cuda_device_id="0").run(sim_dir)
    assert result.dtype == np.float32 and result.ndim == 1
    assert np.all(result == 42.0)
    assert (sim_dir / "genout.dat").exists()
    assert "Simulation completed" in (sim_dir / "fw2_execution.log").read_text()
    assert Launcher().run(sim_dir, load_results=False) == sim_dir / "genout.dat"


def test_run_failure_raises_simulation_error(sim_dir, monkeypatch, no_cuda):
    monkeypatch.setattr(engine_mod, "Engine", _FailingEngine)
    cwd = Path.cwd()
    with pytest.raises(SimulationError):
        Launcher().run(sim_dir)
    assert Path.cwd() == cwd
    assert "simulated CUDA failure" in (sim_dir / "fw2_execution.log").read_text()


def test_run_wrong_dimension_is_a_simulation_error(sim_dir, monkeypatch, no_cuda):
    monkeypatch.setattr(engine_mod, "Engine", _FakeEngine)
    with pytest.raises(SimulationError):
        Launcher(is_3d=True).run(sim_dir)


def test_cpu_mode_not_implemented(sim_dir):
    with pytest.raises(NotImplementedError):
        Launcher(use_gpu=False).run(sim_dir)


def test_missing_inputs_are_a_simulation_error(no_cuda):
    with tempfile.TemporaryDirectory() as td:
        with pytest.raises(SimulationError):
            Launcher().run(Path(td))


@pytest.mark.parametrize("given,expected", [(None, [0]), (2, [2]), ("1", [1]), ("3,4", [3, 4]),
                                            ([5, 6], [5, 6]), (" 7 , 2", [7, 2])])
def test_device_selection(given, expected):
    assert device_list(given) == expected
    assert resolve_device(given) == expected[0]
    la = Launcher(cuda_device_id=given)
    assert la.device_index == expected[0] and la.device_ids == expected
    assert la.cuda_device_id == ",".join(map(str, expected))


def test_several_devices_are_reported_not_silently_dropped(caplog):
    import logging

    with caplog.at_level(logging.WARNING):
        assert resolve_device([3, 1, 2]) == 3
    assert any("one simulation runs on one GPU" in r.getMessage() for r in caplog.records)
    with pytest.raises(ValueError):
        device_list([])
