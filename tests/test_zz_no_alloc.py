"""fw_run_noalloc: the solve that allocates nothing, for callers that cannot call cudaMalloc
while they run (their device memory comes from their own pool, or their device footprint is
fixed after start-up). It keeps the wavefield in a fixed 32 MiB device array inside the library;
the caller passes device inputs and a device output buffer. This file is collected last on
purpose.

Checked here through the C ABI: two calls in a row each match the regular entry point
(fw_create + fw_set_fields + fw_run) within the engine's tolerance (1e-4 relative L2 of the
sensor traces), and a grid larger than the array is rejected with FW_ERR_ARGUMENT.
"""

import ctypes as C

import numpy as np
import pytest

from fdtd_oracle import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


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


def test_noalloc_matches_regular_entry_point_twice(engine_lib, cuda):
    from fullwave25_gb300.engine import Engine, desc_from_inputs, _FP
    from fullwave25_gb300.workloads import plain_2d_inputs

    torch = cuda
    inp = plain_2d_inputs(shape=(200, 168), nt=600, n_pml=20, n_transition=20, seed=5)
    with Engine(inp) as eng:
        ref = eng.run()
    keep = []
    fields = _device_fields(inp, torch, keep)
    desc = desc_from_inputs(inp)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        out = torch.full(ref.shape, float("nan"), dtype=torch.float32, device="cuda")
        st = engine_lib.fw_run_noalloc(C.byref(desc), C.byref(fields), C.c_void_p(stream),
                                       C.cast(C.c_void_p(out.data_ptr()), _FP))
        assert st == 0, engine_lib.fw_last_error(None)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert np.isfinite(got).all()
        err = rel_l2(got, ref)
        assert err < TOL, f"call {call}: rel-L2 {err:.3e} vs fw_run"


def test_noalloc_rejects_grid_beyond_scratch(engine_lib, cuda):
    from fullwave25_gb300.engine import FwDesc, FwFields, _FP

    torch = cuda
    desc = FwDesc(ndim=2, nx=1024, ny=1024, nz=1, nt=10, nt_ic=10, mod_t=1, dx=1e-4, dy=1e-4,
                  dz=0.0, dt=1e-8, c0=1540.0, ncoords=0, ncoordsout=0, ncoordszero=0, ndmap=1,
                  isotropic=1, n_relax=2)
    out = torch.zeros(16, device="cuda")
    st = engine_lib.fw_run_noalloc(C.byref(desc), C.byref(FwFields(on_device=1)), None,
                                   C.cast(C.c_void_p(out.data_ptr()), _FP))
    assert st == 1
    msg = engine_lib.fw_last_error(None).decode()
    assert "maximum" in msg and "33554432" in msg
