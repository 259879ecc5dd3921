"""The batched workload's device-side builder (run here with torch on the CPU) produces exactly
the arrays of the host-side API path (NumPy medium, relaxation lookup, PML builder)."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("i", [0, 5, 11])
def test_device_builder_equals_host_api_build(i):
    from fullwave25_gb300.workloads3d import to_host_inputs
    from fullwave25_gb300.workloads_batch import batch_inputs_host, batch_instance

    kw = dict(scale=0.12, n_pml=10, n_transition=10)
    dev = to_host_inputs(batch_instance(i, device=torch.device("cpu"), **kw))
    host = batch_inputs_host(i, **kw)
    assert tuple(dev.shape) == tuple(host.shape) and dev.nt == host.nt
    assert set(host.maps) <= set(dev.maps)
    for k in host.maps:
        np.testing.assert_array_equal(dev.maps[k], host.maps[k], err_msg=k)
    for k in ("dcmap", "dmap", "icc", "icmat", "outc"):
        np.testing.assert_array_equal(getattr(dev, k), getattr(host, k), err_msg=k)
