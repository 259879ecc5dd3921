"""The C-ABI library builds, loads and exports every symbol include/fwgb.h declares; argument
errors are reported through status codes without touching a GPU."""

import ctypes as C
import re
from pathlib import Path

import pytest

from fullwave25_gb300 import engine

HEADER = Path(__file__).resolve().parent.parent / "include" / "fwgb.h"


def declared_symbols():
    return sorted(set(re.findall(r"FWGB_API\s+(?:const\s+char\s*\*|int)\s*(fw_\w+)\s*\(",
                                 HEADER.read_text())))


def test_header_and_binding_agree():
    assert declared_symbols() == sorted(engine.EXPORTED)


def test_library_exports_every_declared_symbol(engine_lib):
    for name in declared_symbols():
        assert hasattr(engine_lib, name), name
    assert engine_lib.fw_abi_version() == 1


@pytest.mark.parametrize("field,value,code", [
    ("ndim", 4, 1), ("nx", 10, 1), ("mod_t", 0, 1), ("isotropic", 2, 1), ("n_relax", 3, 6),
    ("dt", 0.0, 1), ("ndmap", 65536, 1),   # the device keeps a cell's tap-set index in 16 bits
])
def test_create_rejects_bad_descriptor(engine_lib, field, value, code):
    d = engine.FwDesc(ndim=2, nx=64, ny=64, nz=1, nt=10, nt_ic=10, mod_t=1, dx=1e-4, dy=1e-4,
                      dz=0.0, dt=1e-8, c0=1540.0, ncoords=1, ncoordsout=1, ncoordszero=0,
                      ndmap=1, isotropic=1, n_relax=2)
    setattr(d, field, value)
    h = C.c_void_p()
    assert engine_lib.fw_create(C.byref(d), C.byref(h)) == code
    assert not h.value
    assert engine_lib.fw_last_error(None)


def test_null_handle_is_an_error(engine_lib):
    assert engine_lib.fw_advance(None, None, 1) == 1
    assert engine_lib.fw_destroy(None) == 0
