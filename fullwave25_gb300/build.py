"""Build the engine's shared library ``libfwgb.so`` in-tree with nvcc for sm_103a.

``python -m fullwave25_gb300.build`` (or :func:`build`) compiles ``csrc/*.cu`` into
``fullwave25_gb300/libfwgb.so``. The library exports the C ABI of ``include/fwgb.h`` and links
the CUDA runtime statically, so it loads next to any PyTorch build.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
LIB = PKG / "libfwgb.so"
SOURCES = [PKG / "csrc" / f for f in ("engine.cu", "launch.cu", "group.cu", "adjoint.cu",
                                       "noalloc.cu")]
OBJDIR = PKG / "_build"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def needs_build() -> bool:
    if not LIB.exists():
        return True
    mtime = LIB.stat().st_mtime
    deps = list((PKG / "csrc").glob("*")) + [ROOT / "include" / "fwgb.h"]
    return any(p.stat().st_mtime > mtime for p in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every translation unit in parallel (one nvcc process each), then link."""
    if not force and not needs_build():
        return LIB
    OBJDIR.mkdir(exist_ok=True)
    common = [nvcc_path(), *ARCH, "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "-I", str(ROOT / "include")]
    if verbose:
        common.insert(1, "-Xptxas=-v")
    procs, objs = [], []
    for src in SOURCES:
        obj = OBJDIR / (src.stem + ".o")
        cmd = [*common, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((src, subprocess.Popen(cmd)))
        objs.append(obj)
    failed = [str(src) for src, p in procs if p.wait() != 0]
    if failed:
        raise subprocess.CalledProcessError(1, "nvcc " + " ".join(failed))
    subprocess.run([nvcc_path(), *ARCH, "--shared", "-Xcompiler", "-fPIC", "-o",
                    str(LIB) + ".tmp", *[str(o) for o in objs]], check=True)
    os.replace(str(LIB) + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
