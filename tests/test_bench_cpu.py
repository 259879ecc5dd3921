"""Host-side pieces of bench.py (no GPU): the reference arm's answer for workloads that have no
reference counterpart, and the workload descriptions of the physics variants."""

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_without_counterpart_prints_unavailable():
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--workload", "serve2d"], capture_output=True, text=True, timeout=300,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "serve2d" in line["unavailable"]


def test_workload_descriptions_of_physics_variants():
    sys.path.insert(0, str(ROOT))
    import bench

    iso = bench.workload_desc("plain2d")
    exp = bench.workload_desc("plain2d", physics="exp")
    assert iso["grid"] == [944, 688] and exp["grid"] == [864, 608]
    an3 = bench.workload_desc("plain3d", 112, physics="aniso")
    assert an3["grid"] == [256] * 3 and an3["physics"] == "aniso"
    assert "anisotropic" in an3["workload"]


def test_workload_entry_points_pass_their_arguments(monkeypatch):
    """Every ``--workload`` entry point hands its command-line arguments to its measurement
    (the measurements themselves need a GPU and are replaced by recorders here)."""
    sys.path.insert(0, str(ROOT))
    import bench
    import torch

    calls = {}

    def recorder(name):
        def f(*a, **k):
            calls[name] = (a, k)
            return {"value": 1.0, "config": {}, "host_to_host_s": 1.0}
        return f

    for name in ("measure_adjoint", "measure_adjoint3d", "measure_batch", "measure_serve",
                 "measure_solver3d"):
        monkeypatch.setattr(bench, name, recorder(name))
    monkeypatch.setattr(torch.cuda, "set_device", lambda *a: None)
    argv = ["bench.py", "--steps", "4", "--warmup", "5", "--grid", "96", "--nt", "70",
            "--checkpoint-every", "10", "--batch", "7", "--host-sample", "2", "--solver-sample", "3",
            "--rate", "5", "--duration", "2", "--scale", "0.25"]
    for workload in ("adjoint2d", "adjoint3d", "batch2d", "serve2d", "solver3d"):
        monkeypatch.setattr(sys, "argv", argv + ["--workload", workload])
        bench.main()
    assert calls["measure_adjoint"][0] == (96, 70, 10, 4, 5)
    assert calls["measure_adjoint3d"][0] == (96, 70, 10, 4, 5, "isotropic")
    assert calls["measure_batch"][0] == (7, 4, 5, 2, 3)
    assert calls["measure_serve"][0][:3] == (5.0, 2.0, 0.25)
    assert calls["measure_solver3d"][0] == (96,)
