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
