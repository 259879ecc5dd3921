"""FD coefficient tables against the reference's own values (golden) and the stencil identity."""

import numpy as np
import pytest

from fullwave25_gb300 import coefficients
from golden_io import HERE

G = np.load(HERE / "coeff_tables.npz")


@pytest.mark.parametrize("tag", ["2d", "3d"])
@pytest.mark.parametrize("cfl", [0.05, 0.1, 0.2, 0.3, 0.45])
def test_d_matrix_matches_reference(tag, cfl):
    d = coefficients.d_matrix(cfl, is_3d=tag == "3d")
    np.testing.assert_array_equal(d, G[f"d_{tag}_cfl{cfl}"])


@pytest.mark.parametrize("tag", ["2d", "3d"])
def test_dmap_and_dcmap_match_reference(tag):
    c = G[f"dmap_c_{tag}"]
    dmap = coefficients.d_map(c, float(G[f"dmap_dt_{tag}"]), float(G[f"dmap_dx_{tag}"]),
                              is_3d=tag == "3d")
    np.testing.assert_array_equal(dmap, G[f"dmap_{tag}"])
    np.testing.assert_array_equal(coefficients.dc_map(c), G[f"dcmap_{tag}"])


@pytest.mark.parametrize("is_3d", [False, True])
@pytest.mark.parametrize("cfl", np.linspace(0.02, 0.48, 24))
def test_offaxis_stencil_consistency(is_3d, cfl):
    """sum (2m-1) d[m,0] + 2 (ndim-1) d[1,1] = 1: the table is a consistent first-derivative
    stencil only with one off-axis tap pair per transverse axis, which pins the geometry the
    engine and oracle use for d[1,1]."""
    d = coefficients.d_matrix(float(cfl), is_3d=is_3d)
    assert abs(coefficients.consistency_residual(d, is_3d=is_3d)) < 1e-4
    # the other plausible reading (off-axis pairs not counted) is far from consistent
    m = np.arange(1, 9)
    if cfl > 0.1:
        assert abs(((2 * m - 1) * d[1:9, 0]).sum() - 1.0) > 1e-3


def test_pack_taps_layout():
    dmap = np.arange(18 * 3, dtype=np.float64).reshape(9, 2, 3)
    t = coefficients.pack_taps(dmap)
    assert t.shape == (3, 12)
    np.testing.assert_array_equal(t[:, :8], dmap[1:9, 0, :].T)
    np.testing.assert_array_equal(t[:, 8], dmap[1, 1, :])
    assert not t[:, 9:].any()
