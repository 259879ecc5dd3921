"""ctypes binding of the C ABI in ``include/fwgb.h`` (``libfwgb.so``).

This is the only module that talks to the native library. There is no CPU fallback: if the
library is missing or no CUDA device is present, :func:`load_library` / :class:`Engine` raise.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from .inputs import ISOTROPIC_MAPS, EngineInputs, anisotropic_extra_maps

LIB_PATH = Path(__file__).resolve().parent / "libfwgb.so"

FW_STATUS = {0: "FW_OK", 1: "FW_ERR_ARGUMENT", 2: "FW_ERR_CUDA", 3: "FW_ERR_STATE",
             4: "FW_ERR_OOM", 5: "FW_ERR_DEVICE", 6: "FW_ERR_UNSUPPORTED"}

# every symbol include/fwgb.h declares
EXPORTED = ("fw_abi_version", "fw_create", "fw_set_fields", "fw_set_fields_aniso",
            "fw_set_fields_exp",
            "fw_set_source_signal",
            "fw_set_source_columns", "fw_set_sensor_groups", "fw_run",
            "fw_reset", "fw_advance", "fw_read_traces", "fw_trace_buffer", "fw_get_field",
            "fw_current_step", "fw_device_bytes", "fw_kernel_variant", "fw_block_tile", "fw_selftest_waits", "fw_copy_state_rows",
            "fw_launches_per_step",
            "fw_destroy", "fw_adjoint_forward", "fw_adjoint_backward", "fw_group_create", "fw_group_run", "fw_group_set_members",
            "fw_group_advance", "fw_group_block_tile", "fw_group_destroy",
            "fw_run_noalloc", "fw_last_error")


class FwDesc(C.Structure):
    _fields_ = [("ndim", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32),
                ("nt", C.c_int32), ("nt_ic", C.c_int32), ("mod_t", C.c_int32),
                ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float), ("dt", C.c_float),
                ("c0", C.c_float), ("ncoords", C.c_int32), ("ncoordsout", C.c_int32),
                ("ncoordszero", C.c_int32), ("ndmap", C.c_int32), ("isotropic", C.c_int32),
                ("n_relax", C.c_int32)]


_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int32)


class FwFields(C.Structure):
    _fields_ = [("d", _FP), ("dmap", _FP), ("dcmap", _IP), ("c", _FP), ("rho", _FP), ("K", _FP),
                ("beta", _FP), ("kappax", _FP), ("kappau", _FP),
                ("apmlu1", _FP), ("bpmlu1", _FP), ("apmlx1", _FP), ("bpmlx1", _FP),
                ("apmlu2", _FP), ("bpmlu2", _FP), ("apmlx2", _FP), ("bpmlx2", _FP),
                ("icc", _IP), ("outc", _IP), ("icczero", _IP), ("icmat", _FP),
                ("on_device", C.c_int32)]


# order of the gradient arrays returned by fw_adjoint_backward (isotropic relaxation engine; the
# exponential engine fills dt/rho, dt*K and a_exp in the au1 slot)
ADJOINT_MAPS = ("rdt_rho", "dt_k", "inv_ku", "inv_kx", "au1", "bu1", "au2", "bu2",
                "ax1", "bx1", "ax2", "bx2")


def adjoint_gradient_maps(inputs) -> tuple:
    """Engine-map names of ``fw_adjoint_backward``'s gradient arrays, in output order:
    ``ADJOINT_MAPS`` (12), or for the anisotropic engine 2 + 10 ndim: dt/rho, dt*K, then per
    derivative axis 1/kappa, a1, b1, a2, b2 of the pressure-gradient maps (u, w, v), then the
    same of the velocity-divergence maps (x, y, z); followed by ``beta2dt`` (2 dt beta) when the
    beta map is not zero everywhere."""
    beta = inputs.maps.get("beta")
    tail = ("beta2dt",) if beta is not None and bool((beta != 0).any()) else ()
    if "kappay" not in inputs.maps:
        return ADJOINT_MAPS + tail
    names = ["rdt_rho", "dt_k"]
    for letters in ("uwv", "xyz"):
        for a in range(len(inputs.shape)):
            g = letters[a]
            names += [f"inv_k{g}", f"a{g}1", f"b{g}1", f"a{g}2", f"b{g}2"]
    return tuple(names) + tail


ANISO_FIELDS = tuple(f"{k}{ax}{nu}" if k != "kappa" else f"kappa{ax}"
                     for ax in ("w", "y", "v", "z")
                     for k, nu in (("kappa", ""), ("apml", 1), ("bpml", 1), ("apml", 2), ("bpml", 2)))


class FwFieldsAniso(C.Structure):
    _fields_ = [(n, _FP) for n in ANISO_FIELDS]


class EngineError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, call: str, status: int, message: str) -> None:
        super().__init__(f"{call} -> {FW_STATUS.get(status, status)}: {message}")
        self.status = status


_lib = None


def load_library(path: Path | None = None) -> C.CDLL:
    """Load ``libfwgb.so`` and declare its signatures; raises if it is not built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is missing: build the CUDA engine first (python -m fullwave25_gb300.build)")
    lib = C.CDLL(str(p))
    vp = C.c_void_p
    H = C.c_void_p
    sig = {
        "fw_abi_version": (C.c_int, []),
        "fw_create": (C.c_int, [C.POINTER(FwDesc), C.POINTER(H)]),
        "fw_set_fields": (C.c_int, [H, C.POINTER(FwFields)]),
        "fw_set_fields_aniso": (C.c_int, [H, C.POINTER(FwFields), C.POINTER(FwFieldsAniso)]),
        "fw_set_fields_exp": (C.c_int, [H, C.POINTER(FwFields), _FP]),
        "fw_set_source_signal": (C.c_int, [H, _FP, C.c_int32]),
        "fw_set_source_columns": (C.c_int, [H, vp, _FP, C.c_int32, C.c_int32, C.c_int32]),
        "fw_set_sensor_groups": (C.c_int, [H, _IP, _FP, C.c_int32]),
        "fw_run": (C.c_int, [H, vp, _FP, C.c_int32]),
        "fw_reset": (C.c_int, [H, vp]),
        "fw_advance": (C.c_int, [H, vp, C.c_int32]),
        "fw_read_traces": (C.c_int, [H, vp, C.c_int32, C.c_int32, _FP, C.c_int32]),
        "fw_trace_buffer": (C.c_int, [H, C.POINTER(_FP)]),
        "fw_get_field": (C.c_int, [H, vp, C.c_int32, _FP, C.c_int32]),
        "fw_current_step": (C.c_int, [H, _IP]),
        "fw_device_bytes": (C.c_int, [H, C.POINTER(C.c_uint64)]),
        "fw_kernel_variant": (C.c_int, [H, _IP]),
        "fw_block_tile": (C.c_int, [H, _IP]),
        "fw_selftest_waits": (C.c_int, [_IP]),
        "fw_copy_state_rows": (C.c_int, [H, C.c_int32, H, C.c_int32, C.c_int32, vp]),
        "fw_launches_per_step": (C.c_int, [H, _IP]),
        "fw_destroy": (C.c_int, [H]),
        "fw_adjoint_forward": (C.c_int, [H, vp, C.c_int32]),
        "fw_adjoint_backward": (C.c_int, [H, vp, _FP, C.POINTER(C.c_double)]),
        "fw_group_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]),
        "fw_group_run": (C.c_int, [C.c_void_p, vp]),
        "fw_group_set_members": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p), C.c_int32]),
        "fw_group_advance": (C.c_int, [C.c_void_p, vp, C.c_int32]),
        "fw_group_block_tile": (C.c_int, [C.c_void_p, _IP]),
        "fw_group_destroy": (C.c_int, [C.c_void_p]),
        "fw_run_noalloc": (C.c_int, [C.POINTER(FwDesc), C.POINTER(FwFields), vp, _FP]),
        "fw_last_error": (C.c_char_p, [H]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _fp(a):
    return a.ctypes.data_as(_FP) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(_IP) if a is not None else None


def _c_f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _c_i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def desc_from_inputs(inp) -> FwDesc:
    nz = inp.shape[2] if inp.ndim == 3 else 1
    dz = inp.spacing[2] if inp.ndim == 3 else 0.0
    return FwDesc(ndim=inp.ndim, nx=inp.shape[0], ny=inp.shape[1], nz=nz, nt=inp.nt,
                  nt_ic=int(inp.icmat.shape[1]), mod_t=inp.mod_t, dx=inp.spacing[0],
                  dy=inp.spacing[1], dz=dz,
                  dt=inp.dt, c0=inp.c0, ncoords=inp.icc.shape[0], ncoordsout=inp.outc.shape[0],
                  ncoordszero=inp.icczero.shape[0], ndmap=inp.dmap.shape[2],
                  isotropic=int("kappay" not in inp.maps),
                  n_relax=0 if "a_exp" in inp.maps else 2)


class Engine:
    """One simulation on the current CUDA device, driven through the C ABI."""

    def __init__(self, inputs, *, validate: bool = True) -> None:
        if validate and isinstance(inputs, EngineInputs):
            inputs.validate()
        self.lib = load_library()
        self.inputs = inputs
        self.desc = desc_from_inputs(inputs)
        self._h = C.c_void_p()
        self._check("fw_create", self.lib.fw_create(C.byref(self.desc), C.byref(self._h)), None)
        try:
            self.set_fields(inputs)
        except Exception:
            self.close()
            raise

    # -- plumbing -----------------------------------------------------------------------------
    def _check(self, call: str, status: int, handle) -> None:
        if status != 0:
            msg = self.lib.fw_last_error(handle)
            raise EngineError(call, status, msg.decode() if msg else "")

    def _call(self, name: str, *args) -> None:
        self._check(name, getattr(self.lib, name)(self._h, *args), self._h)

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def set_fields(self, inp) -> None:
        if not isinstance(inp, EngineInputs):
            return self._set_device_fields(inp)
        keep = {}  # holds the contiguous copies alive during the call

        def f(name, arr, conv):
            keep[name] = conv(arr)
            return keep[name]

        m = inp.maps
        fields = FwFields(
            d=_fp(f("d", inp.d, _c_f32)), dmap=_fp(f("dmap", inp.dmap, _c_f32)),
            dcmap=_ip(f("dcmap", inp.dcmap, _c_i32)), on_device=0,
            icc=_ip(f("icc", inp.icc, _c_i32)), outc=_ip(f("outc", inp.outc, _c_i32)),
            icczero=_ip(f("icczero", inp.icczero, _c_i32)),
            icmat=_fp(f("icmat", inp.icmat, _c_f32)),
            **{k: _fp(f(k, m[k], _c_f32)) for k in ("c", "rho", "K", "beta", *ISOTROPIC_MAPS)
               if k in m},
        )
        if "a_exp" in m:
            self._call("fw_set_fields_exp", C.byref(fields), _fp(f("a_exp", m["a_exp"], _c_f32)))
        elif inp.isotropic:
            self._call("fw_set_fields", C.byref(fields))
        else:
            an = FwFieldsAniso(**{k: _fp(f(k, m[k], _c_f32))
                                  for k in anisotropic_extra_maps(inp.ndim)})
            self._call("fw_set_fields_aniso", C.byref(fields), C.byref(an))

    def _set_device_fields(self, inp) -> None:
        """Fields given as CUDA tensors (``workloads3d.DeviceInputs``): no host round trip."""
        import torch  # noqa: PLC0415

        dev = inp.maps["rho"].device
        keep = {"d": torch.as_tensor(np.ascontiguousarray(inp.d, np.float32), device=dev),
                "dmap": torch.as_tensor(np.ascontiguousarray(inp.dmap, np.float32), device=dev)}
        fptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), _FP) if t.numel() else None  # noqa: E731
        iptr = lambda t: C.cast(C.c_void_p(t.data_ptr()), _IP) if t.numel() else None  # noqa: E731
        m = inp.maps
        exp = "a_exp" in m   # exponential-attenuation engine: no relaxation maps
        names = ("c", "rho", "K", "beta", *(("a_exp",) if exp else ISOTROPIC_MAPS))
        for k in names:
            assert m[k].dtype == torch.float32 and m[k].is_contiguous() and m[k].is_cuda, k
        fields = FwFields(
            d=fptr(keep["d"]), dmap=fptr(keep["dmap"]), dcmap=iptr(inp.dcmap),
            icc=iptr(inp.icc), outc=iptr(inp.outc), icczero=iptr(inp.icczero),
            icmat=fptr(inp.icmat), on_device=1,
            **{k: fptr(m[k]) for k in names if k != "a_exp"})
        # the tensors were produced on the caller's current stream: wait for that stream only,
        # so that work on other streams (other simulations) keeps running
        torch.cuda.current_stream(dev).synchronize()
        if exp:
            self._call("fw_set_fields_exp", C.byref(fields), fptr(m["a_exp"]))
        elif "kappay" in m:
            for k in anisotropic_extra_maps(inp.ndim):
                assert m[k].dtype == torch.float32 and m[k].is_contiguous() and m[k].is_cuda, k
            an = FwFieldsAniso(**{k: fptr(m[k]) for k in anisotropic_extra_maps(inp.ndim)})
            self._call("fw_set_fields_aniso", C.byref(fields), C.byref(an))
        else:
            self._call("fw_set_fields", C.byref(fields))

    def set_source_columns(self, cols: np.ndarray, n0: int, stream: int | None = None) -> None:
        """Upload source samples of steps ``[n0, n0 + len(cols))`` (time-major, host)."""
        a = np.ascontiguousarray(cols, dtype=np.float32)
        self._call("fw_set_source_columns", C.c_void_p(stream or 0), _fp(a), int(n0),
                   int(a.shape[0]), 0)

    def read_traces_to(self, dst: np.ndarray, row0: int, stream: int | None = None) -> None:
        """Copy trace rows ``[row0, row0 + len(dst))`` into the host array ``dst``."""
        assert dst.dtype == np.float32 and dst.flags.c_contiguous
        self._call("fw_read_traces", C.c_void_p(stream or 0), int(row0), int(dst.shape[0]),
                   _fp(dst), 0)

    def set_sensor_groups(self, group_of_sensor, weight, n_groups: int) -> None:
        """Record weighted sums per sensor group (traces become ``[n_out, n_groups]``)."""
        g = _c_i32(group_of_sensor)
        w = _c_f32(weight)
        if g.shape != (self.inputs.outc.shape[0],) or w.shape != g.shape:
            raise ValueError("one group id and one weight per sensor")
        self._call("fw_set_sensor_groups", _ip(g), _fp(w), int(n_groups))
        self._n_cols = int(n_groups) or self.inputs.outc.shape[0]

    @property
    def n_cols(self) -> int:
        return getattr(self, "_n_cols", self.inputs.outc.shape[0])

    def set_source_signal(self, icmat: np.ndarray) -> None:
        a = _c_f32(icmat)
        if a.shape != self.inputs.icmat.shape:
            raise ValueError(f"icmat must be {self.inputs.icmat.shape}, got {a.shape}")
        self._call("fw_set_source_signal", _fp(a), 0)

    # -- stepping -----------------------------------------------------------------------------
    @property
    def n_out(self) -> int:
        return self.inputs.n_out

    def run(self, stream: int | None = None) -> np.ndarray:
        """Full solve; returns the float32 traces ``[n_out, ncoordsout]`` (genout layout)."""
        out = np.empty((self.n_out, self.n_cols), dtype=np.float32)
        self._call("fw_run", C.c_void_p(stream or 0), _fp(out), 0)
        return out

    def run_into(self, dev_ptr: int, stream: int | None = None) -> None:
        """Full solve writing the traces into device memory at ``dev_ptr`` (asynchronous)."""
        self._call("fw_run", C.c_void_p(stream or 0), C.cast(C.c_void_p(dev_ptr), _FP), 1)

    def reset(self, stream: int | None = None) -> None:
        self._call("fw_reset", C.c_void_p(stream or 0))

    def advance(self, n_steps: int, stream: int | None = None) -> None:
        self._call("fw_advance", C.c_void_p(stream or 0), int(n_steps))

    def read_traces(self, row0: int = 0, n_rows: int | None = None,
                    stream: int | None = None) -> np.ndarray:
        n_rows = self.n_out - row0 if n_rows is None else n_rows
        out = np.empty((n_rows, self.n_cols), dtype=np.float32)
        self._call("fw_read_traces", C.c_void_p(stream or 0), int(row0), int(n_rows), _fp(out), 0)
        return out

    def read_traces_into(self, row0: int, n_rows: int, dev_ptr: int,
                         stream: int | None = None) -> None:
        self._call("fw_read_traces", C.c_void_p(stream or 0), int(row0), int(n_rows),
                   C.cast(C.c_void_p(dev_ptr), _FP), 1)

    def trace_buffer(self) -> int:
        p = _FP()
        self._call("fw_trace_buffer", C.byref(p))
        return C.cast(p, C.c_void_p).value

    def get_field(self, field: int = 0, stream: int | None = None) -> np.ndarray:
        out = np.empty(self.inputs.shape, dtype=np.float32)
        self._call("fw_get_field", C.c_void_p(stream or 0), int(field), _fp(out), 0)
        return out

    def adjoint_forward(self, checkpoint_every: int, stream: int | None = None) -> None:
        self._call("fw_adjoint_forward", C.c_void_p(stream or 0), int(checkpoint_every))

    def adjoint_backward(self, residual_ptr: int, grad_ptr: int, stream: int | None = None) -> None:
        """``residual_ptr``: device float32 [n_out, ncoordsout]; ``grad_ptr``: device float64
        [n, *shape], n and order as ``adjoint_gradient_maps(inputs)``."""
        self._call("fw_adjoint_backward", C.c_void_p(stream or 0),
                   C.cast(C.c_void_p(residual_ptr), _FP),
                   C.cast(C.c_void_p(grad_ptr), C.POINTER(C.c_double)))

    @property
    def current_step(self) -> int:
        v = C.c_int32()
        self._call("fw_current_step", C.byref(v))
        return v.value

    @property
    def device_bytes(self) -> int:
        v = C.c_uint64()
        self._call("fw_device_bytes", C.byref(v))
        return v.value

    @property
    def kernel_variant(self) -> str:
        v = C.c_int32()
        self._call("fw_kernel_variant", C.byref(v))
        return {0: "direct", 1: "march", 2: "persistent", 3: "stream", 4: "tile"}[v.value]

    def copy_state_rows_from(self, src: "Engine", src_row0: int, dst_row0: int, n_rows: int,
                             stream: int | None = None) -> None:
        """Copy ``n_rows`` depth rows of every state field from ``src`` (same cross-section)."""
        st = self.lib.fw_copy_state_rows(self._h, int(dst_row0), src.handle, int(src_row0),
                                         int(n_rows), C.c_void_p(stream or 0))
        self._check("fw_copy_state_rows", st, self._h)

    @property
    def block_tile(self) -> tuple:
        """Cells per block of the kernels in use along (x, y, z); 2D handles report the shape
        the autotuner picked once the first advance from step 0 has run."""
        v = (C.c_int32 * 3)()
        self._call("fw_block_tile", v)
        return tuple(v)

    @property
    def launches_per_step(self) -> int:
        v = C.c_int32()
        self._call("fw_launches_per_step", C.byref(v))
        return v.value

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self.lib.fw_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def selftest_waits() -> tuple:
    """Run the bounded-wait self-test (``fw_selftest_waits``): returns the status words of the
    mbarrier-wait kernel and of the grid-barrier kernel, each of which waits on something that
    never completes and must give up (expected ``(0x1, 0x4)``)."""
    lib = load_library()
    out = (C.c_int32 * 2)()
    st = lib.fw_selftest_waits(out)
    if st:
        raise EngineError("fw_selftest_waits", st, lib.fw_last_error(None).decode())
    return int(out[0]), int(out[1])


class EngineGroup:
    """Many 2D simulations stepped together (``fw_group_*``): one launch per phase per step."""

    def __init__(self, engines):
        self.engines = list(engines)
        self.lib = load_library()
        arr = (C.c_void_p * len(self.engines))(*[e.handle.value for e in self.engines])
        self._g = C.c_void_p()
        st = self.lib.fw_group_create(arr, len(self.engines), C.byref(self._g))
        if st:
            raise EngineError("fw_group_create", st, self.lib.fw_last_error(None).decode())

    def run(self, stream: int | None = None) -> None:
        st = self.lib.fw_group_run(self._g, C.c_void_p(stream or 0))
        if st:
            raise EngineError("fw_group_run", st, self.lib.fw_last_error(None).decode())

    def set_members(self, engines) -> None:
        self.engines = list(engines)
        arr = (C.c_void_p * max(1, len(self.engines)))(*[e.handle.value for e in self.engines])
        st = self.lib.fw_group_set_members(self._g, arr, len(self.engines))
        if st:
            raise EngineError("fw_group_set_members", st, self.lib.fw_last_error(None).decode())

    def advance(self, n_steps: int, stream: int | None = None) -> None:
        st = self.lib.fw_group_advance(self._g, C.c_void_p(stream or 0), int(n_steps))
        if st:
            raise EngineError("fw_group_advance", st, self.lib.fw_last_error(None).decode())

    def traces(self) -> list:
        return [e.read_traces() for e in self.engines]

    @property
    def block_tile(self) -> tuple:
        """Cells per block of the group's kernels along (x, y, z)."""
        v = (C.c_int32 * 3)()
        st = self.lib.fw_group_block_tile(self._g, v)
        if st:
            raise EngineError("fw_group_block_tile", st, "")
        return tuple(v)

    def close(self) -> None:
        if getattr(self, "_g", None) and self._g.value:
            self.lib.fw_group_destroy(self._g)
            self._g = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
