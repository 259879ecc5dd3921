"""Whole-domain output reshapes and the display compression (host side, no GPU)."""

from types import SimpleNamespace

import numpy as np
import pytest

from fullwave25_gb300.signal_process import (reshape_whole_sensor_to_nt_nx_ny,
                                             reshape_whole_sensor_to_nt_nx_ny_nz,
                                             reshape_whole_sensor_to_nx_ny_nt,
                                             signed_power_compression)


def _whole(nx, ny, nt, nz=None):
    """Traces of a whole-domain recording: sensor k in C order of the grid, value encodes
    (t, i, j[, l])."""
    idx = np.argwhere(np.ones((nx, ny) if nz is None else (nx, ny, nz), dtype=bool))
    t = np.arange(nt)
    code = idx @ (np.array([10000, 100]) if nz is None else np.array([1000000, 10000, 100]))
    return (code[:, None] + t[None, :] * 1e8).astype(np.float64), idx


def test_nt_nx_ny_indexing():
    out, _ = _whole(5, 7, 3)
    g = SimpleNamespace(nx=5, ny=7)
    a = reshape_whole_sensor_to_nt_nx_ny(out, g)
    assert a.shape == (3, 5, 7)
    assert a[2, 4, 6] == 2e8 + 4 * 10000 + 6 * 100
    b = reshape_whole_sensor_to_nt_nx_ny(out, nx=5, ny=7, use_grid=False)
    np.testing.assert_array_equal(a, b)
    with pytest.raises(ValueError):
        reshape_whole_sensor_to_nt_nx_ny(out, g, nx=5, ny=7)
    with pytest.raises(ValueError):
        reshape_whole_sensor_to_nt_nx_ny(out, nx=5, use_grid=False)


def test_nt_nx_ny_nz_indexing():
    out, _ = _whole(3, 4, 2, nz=5)
    a = reshape_whole_sensor_to_nt_nx_ny_nz(out, SimpleNamespace(nx=3, ny=4, nz=5))
    assert a.shape == (2, 3, 4, 5)
    assert a[1, 2, 3, 4] == 1e8 + 2 * 1000000 + 3 * 10000 + 4 * 100


def test_nx_ny_nt_follows_the_ny_nx_split():
    out = np.arange(6 * 4 * 2, dtype=np.float64).reshape(24, 2)
    a = reshape_whole_sensor_to_nx_ny_nt(out, SimpleNamespace(nx=6, ny=4))
    assert a.shape == (6, 4, 2)
    # sensor axis read as (ny, nx): element (i, j) is sensor j * nx + i
    assert a[5, 3, 1] == out[3 * 6 + 5, 1]


def test_signed_power_compression():
    x = np.array([-8.0, -1.0, 0.0, 1.0, 27.0])
    np.testing.assert_allclose(signed_power_compression(x), [-2.0, -1.0, 0.0, 1.0, 3.0])
    np.testing.assert_allclose(signed_power_compression(x, 1.0), x)
