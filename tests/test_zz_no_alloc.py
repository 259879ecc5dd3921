"""fw_run_noalloc: the solve that allocates nothing, for callers that cannot call cudaMalloc
while they run (their device memory comes from their own pool, or their device footprint is
fixed after start-up). It keeps the wavefield, the derived coefficient maps and the tap table in
a fixed 48 MiB device array inside the library; the caller passes device inputs and a device
output buffer. This file is collected last on purpose.

Checked here through the C ABI:
* two calls in a row each give the regular entry point's traces (fw_create + fw_set_fields +
  fw_run) bit for bit, and the FP64 oracle's within the engine's tolerance (1e-4 relative L2):
  on a plain medium (beta = 0, no air cells, every step recorded) and on the golden case with
  beta, air cells and a recording interval of 3 steps;
* a cell listed twice as a source is driven by its last entry, as in the regular entry point;
* an out-of-grid source, sensor or air coordinate, or a tap index outside the table, is rejected
  with FW_ERR_ARGUMENT before any time step (the output buffer is left untouched, and the
  coordinates used lie just past an edge, where an unchecked write would land inside the
  library's array and show up as wrong values rather than as a fault);
* a grid larger than the array is rejected with FW_ERR_ARGUMENT.
"""

import copy
import ctypes as C

import numpy as np
import pytest

from fdtd_oracle import rel_l2
from fdtd_oracle_c import run_oracle_c as run_oracle
from golden_io import load_case_inputs

pytestmark = pytest.mark.gpu
TOL = 1e-4
FW_ERR_ARGUMENT = 1


def _device_fields(inp, torch, keep):
    from fullwave25_gb300.engine import FwFields, _FP, _IP
    from fullwave25_gb300.inputs import ISOTROPIC_MAPS

    def dev(a, dtype):
        t = torch.as_tensor(np.ascontiguousarray(a, dtype=dtype), device="cuda")
        keep.append(t)
        return t

    fp = lambda t: C.cast(C.c_void_p(t.data_ptr()), _FP) if t.numel() else None  # noqa: E731
    ip = lambda t: C.cast(C.c_void_p(t.data_ptr()), _IP) if t.numel() else None  # noqa: E731
    return FwFields(
        d=fp(dev(inp.d, np.float32)), dmap=fp(dev(inp.dmap, np.float32)),
        dcmap=ip(dev(inp.dcmap, np.int32)), icc=ip(dev(inp.icc, np.int32)),
        outc=ip(dev(inp.outc, np.int32)), icczero=ip(dev(inp.icczero, np.int32)),
        icmat=fp(dev(inp.icmat, np.float32)), on_device=1,
        **{k: fp(dev(inp.maps[k], np.float32)) for k in ("c", "rho", "K", "beta", *ISOTROPIC_MAPS)})


def _noalloc(engine_lib, torch, inp, shape):
    """One call; returns (status, traces as numpy, error text)."""
    from fullwave25_gb300.engine import _FP, desc_from_inputs

    keep = []
    fields = _device_fields(inp, torch, keep)
    desc = desc_from_inputs(inp)
    out = torch.full(shape, float("nan"), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = engine_lib.fw_run_noalloc(C.byref(desc), C.byref(fields), C.c_void_p(stream),
                                   C.cast(C.c_void_p(out.data_ptr()), _FP))
    torch.cuda.synchronize()
    return st, out.cpu().numpy(), engine_lib.fw_last_error(None).decode()


def _plain():
    from fullwave25_gb300.workloads import plain_2d_inputs

    return plain_2d_inputs(shape=(200, 168), nt=600, n_pml=20, n_transition=20, seed=5)


@pytest.mark.parametrize("case", ["plain", "2d_air_beta"])
def test_noalloc_equals_regular_entry_point_twice(engine_lib, cuda, case):
    from fullwave25_gb300.engine import Engine

    inp = _plain() if case == "plain" else load_case_inputs(case)
    if case == "2d_air_beta":
        assert inp.icczero.shape[0] > 0 and np.abs(inp.maps["beta"]).max() > 0 and inp.mod_t > 1
    with Engine(inp) as eng:
        ref = eng.run()
    oracle = run_oracle(inp)
    for call in range(2):
        st, got, msg = _noalloc(engine_lib, cuda, inp, ref.shape)
        assert st == 0, msg
        np.testing.assert_array_equal(got, ref, err_msg=f"call {call}: differs from fw_run")
        err = rel_l2(got, oracle)
        assert err < TOL, f"call {call}: rel-L2 {err:.3e} vs the FP64 oracle"


def test_noalloc_duplicate_source_last_entry_wins(engine_lib, cuda):
    from fullwave25_gb300.engine import Engine

    inp = copy.copy(_plain())
    k = inp.icc.shape[0]
    # the first five sources listed again at the end with other signals: those entries drive
    inp.icc = np.concatenate([inp.icc, inp.icc[:5]]).astype(np.int32)
    inp.icmat = np.concatenate([inp.icmat, -0.5 * inp.icmat[:5, ::-1]]).astype(np.float32)
    assert inp.icc.shape[0] == k + 5
    with Engine(inp) as eng:
        ref = eng.run()
    st, got, msg = _noalloc(engine_lib, cuda, inp, ref.shape)
    assert st == 0, msg
    np.testing.assert_array_equal(got, ref)
    assert rel_l2(got, run_oracle(inp)) < TOL


@pytest.mark.parametrize("what", ["outc", "icc", "icczero", "dcmap"])
def test_noalloc_rejects_out_of_range_indices_before_stepping(engine_lib, cuda, what):
    inp = copy.copy(load_case_inputs("2d_air_beta"))
    nx, ny = inp.shape
    n_out = inp.n_out
    if what == "outc":
        inp.outc = inp.outc.copy()
        inp.outc[3] = (nx, 10)          # one row past the last: inside the array if unchecked
    elif what == "icc":
        inp.icc = inp.icc.copy()
        inp.icc[0] = (10, ny)           # one column past the last
    elif what == "icczero":
        inp.icczero = inp.icczero.copy()
        inp.icczero[2] = (-1, 20)
    else:
        inp.dcmap = inp.dcmap.copy()
        inp.dcmap[nx // 2, ny // 2] = inp.dmap.shape[2]
    st, got, msg = _noalloc(engine_lib, cuda, inp, (n_out, inp.outc.shape[0]))
    assert st == FW_ERR_ARGUMENT, msg
    assert what in msg, msg
    assert np.isnan(got).all()        # no time step ran, nothing was recorded
    # the context and the array are still usable
    good = load_case_inputs("2d_air_beta")
    st, got, msg = _noalloc(engine_lib, cuda, good, (good.n_out, good.outc.shape[0]))
    assert st == 0, msg
    assert rel_l2(got, run_oracle(good)) < TOL


def test_noalloc_rejects_grid_beyond_scratch(engine_lib, cuda):
    from fullwave25_gb300.engine import FwDesc, FwFields, _FP

    torch = cuda
    desc = FwDesc(ndim=2, nx=1024, ny=1024, nz=1, nt=10, nt_ic=10, mod_t=1, dx=1e-4, dy=1e-4,
                  dz=0.0, dt=1e-8, c0=1540.0, ncoords=0, ncoordsout=0, ncoordszero=0, ndmap=1,
                  isotropic=1, n_relax=2)
    out = torch.zeros(16, device="cuda")
    st = engine_lib.fw_run_noalloc(C.byref(desc), C.byref(FwFields(on_device=1)), None,
                                   C.cast(C.c_void_p(out.data_ptr()), _FP))
    assert st == FW_ERR_ARGUMENT
    msg = engine_lib.fw_last_error(None).decode()
    assert "maximum" in msg and "50331648" in msg
