"""ctypes wrapper of the FP64 C oracle (``oracle/fdtd_oracle.c``).

TEST INFRASTRUCTURE ONLY (see the C file's header). ``build()`` compiles the shared object into
``oracle/_build/`` with gcc and OpenMP; ``run_oracle_c(inputs)`` mirrors
``fdtd_oracle.run_oracle`` and returns FP64 traces ``[n_out, ncoordsout]``.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "fdtd_oracle.c"
LIB = HERE / "_build" / "libfdtd_oracle.so"

_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int32)
_DP = C.POINTER(C.c_double)


class OracleDesc(C.Structure):
    _fields_ = [("ndim", C.c_int), ("n", C.c_int64 * 3), ("h", C.c_double * 3), ("dt", C.c_double),
                ("nt", C.c_int), ("nt_ic", C.c_int), ("mod_t", C.c_int), ("ncoords", C.c_int),
                ("ncoordsout", C.c_int), ("ncoordszero", C.c_int), ("ndmap", C.c_int),
                ("dmap", _FP), ("dcmap", _IP), ("rho", _FP), ("K", _FP), ("beta", _FP),
                ("kappau", _FP * 3), ("kappax", _FP * 3), ("au", (_FP * 2) * 3),
                ("bu", (_FP * 2) * 3), ("ax", (_FP * 2) * 3), ("bx", (_FP * 2) * 3),
                ("icc", _IP), ("outc", _IP), ("icczero", _IP), ("icmat", _FP), ("a_exp", _FP)]


def build(force: bool = False) -> Path:
    if LIB.exists() and not force and LIB.stat().st_mtime > SRC.stat().st_mtime:
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    tmp = str(LIB) + f".{os.getpid()}.tmp"
    subprocess.run(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-shared", "-fPIC",
                    "-o", tmp, str(SRC), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(build()))
        lib.oracle_create.restype = C.c_void_p
        lib.oracle_create.argtypes = [C.POINTER(OracleDesc)]
        lib.oracle_run.argtypes = [C.c_void_p, C.c_int, _DP]
        lib.oracle_destroy.argtypes = [C.c_void_p]
        _lib = lib
    return _lib


class OracleC:
    """FP64 C time loop over an ``EngineInputs`` (float32 inputs promoted to float64)."""

    def __init__(self, inp):
        inp.validate()
        self.inp = inp
        f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)  # noqa: E731
        m = inp.maps
        self._keep = k = {
            "dmap": f32(inp.dmap), "dcmap": i32(inp.dcmap), "icc": i32(inp.icc),
            "outc": i32(inp.outc), "icczero": i32(inp.icczero), "icmat": f32(inp.icmat),
            **{n: f32(v) for n, v in m.items() if n not in ("c",)}}
        iso = "kappay" not in m
        gl = ["u"] * 3 if iso else ["u", "w", "v"]
        dl = ["x"] * 3 if iso else ["x", "y", "z"]
        nd = inp.ndim
        exp = "a_exp" in m
        if exp:  # the exponential engine has no relaxation maps; pass the K map as filler
            for ax in ("u", "x"):
                k[f"kappa{ax}"] = k[f"apml{ax}1"] = k[f"apml{ax}2"] = k["K"]
                k[f"bpml{ax}1"] = k[f"bpml{ax}2"] = k["K"]
        fp = lambda a: a.ctypes.data_as(_FP)  # noqa: E731
        ip = lambda a: a.ctypes.data_as(_IP) if a.size else None  # noqa: E731
        shape = list(inp.shape) + [1] * (3 - inp.ndim)
        hs = [float(np.float32(s)) for s in inp.spacing] + [1.0] * (3 - inp.ndim)
        d = OracleDesc(ndim=inp.ndim, n=(C.c_int64 * 3)(*shape), h=(C.c_double * 3)(*hs),
                       dt=float(np.float32(inp.dt)), nt=inp.nt, nt_ic=inp.nt_ic, mod_t=inp.mod_t,
                       ncoords=inp.icc.shape[0], ncoordsout=inp.outc.shape[0],
                       ncoordszero=inp.icczero.shape[0], ndmap=inp.dmap.shape[2],
                       dmap=fp(k["dmap"]), dcmap=ip(k["dcmap"]), rho=fp(k["rho"]), K=fp(k["K"]),
                       beta=fp(k["beta"]),
                       kappau=(_FP * 3)(*[fp(k[f"kappa{gl[a]}"]) for a in range(nd)]),
                       kappax=(_FP * 3)(*[fp(k[f"kappa{dl[a]}"]) for a in range(nd)]),
                       au=((_FP * 2) * 3)(*[(_FP * 2)(fp(k[f"apml{gl[a]}1"]), fp(k[f"apml{gl[a]}2"]))
                                           for a in range(nd)]),
                       bu=((_FP * 2) * 3)(*[(_FP * 2)(fp(k[f"bpml{gl[a]}1"]), fp(k[f"bpml{gl[a]}2"]))
                                           for a in range(nd)]),
                       ax=((_FP * 2) * 3)(*[(_FP * 2)(fp(k[f"apml{dl[a]}1"]), fp(k[f"apml{dl[a]}2"]))
                                           for a in range(nd)]),
                       bx=((_FP * 2) * 3)(*[(_FP * 2)(fp(k[f"bpml{dl[a]}1"]), fp(k[f"bpml{dl[a]}2"]))
                                           for a in range(nd)]),
                       icc=ip(k["icc"]), outc=ip(k["outc"]), icczero=ip(k["icczero"]),
                       icmat=fp(k["icmat"]), a_exp=fp(k["a_exp"]) if exp else None)
        self._desc = d
        self.lib = _load()
        self.h = self.lib.oracle_create(C.byref(d))
        if not self.h:
            raise MemoryError("oracle_create failed")
        self.steps = 0
        self.traces = np.zeros((inp.n_out, inp.outc.shape[0]))

    def run(self, n_steps=None):
        """Advance ``n_steps`` (default: to nT); returns the traces recorded so far."""
        n_steps = self.inp.nt - self.steps if n_steps is None else n_steps
        if self.steps + n_steps > self.inp.nt:
            raise ValueError("cannot step past nT")
        self.lib.oracle_run(self.h, int(n_steps), self.traces.ctypes.data_as(_DP))
        self.steps += n_steps
        return self.traces[: (self.steps + self.inp.mod_t - 1) // self.inp.mod_t].copy()

    def close(self):
        if self.h:
            self.lib.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def run_oracle_c(inputs, n_steps=None) -> np.ndarray:
    o = OracleC(inputs)
    try:
        return o.run(n_steps)
    finally:
        o.close()
