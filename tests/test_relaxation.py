"""Relaxation-table lookup semantics (fullwave/utils/relaxation_parameters.py:18-242), with the
same kind of temporary table the reference's own tests build
(tests/utils/test_relaxation_parameters.py:19-29, :120-191)."""

import numpy as np
from scipy.io import savemat

from fullwave25_gb300.medium import relaxation_param_keys
from fullwave25_gb300.relaxation import RelaxationTable, synthetic_table


def _table(tmp_path):
    alpha = np.array([[0.0, 0.5, 1.0]])
    power = np.array([[0.5, 1.0, 1.5]])
    db = np.zeros((3, 3, 10))
    for i in range(3):
        for j in range(3):
            db[i, j, :] = 100 * i + 10 * j + np.arange(10)
    path = tmp_path / "lut.mat"
    savemat(path, {"database": db, "alpha_0_list": alpha, "power_list": power,
                   "invalid_matrix": np.zeros((3, 3))})
    return RelaxationTable.from_mat(path)


def test_nearest_bin_by_searchsorted(tmp_path):
    t = _table(tmp_path)
    out = t.lookup(np.array([[0.0, 0.2, 0.5, 0.7]]), np.array([[0.5, 0.9, 1.0, 1.2]]))
    # searchsorted(left): 0.2 -> bin 1, 0.7 -> bin 2, 0.9 -> bin 1, 1.2 -> bin 2
    np.testing.assert_array_equal(out["kappa_x1"], [[0, 110, 110, 220]])
    assert list(out) == relaxation_param_keys(2)


def test_out_of_range_is_clipped(tmp_path):
    t = _table(tmp_path)
    out = t.lookup(np.array([[-1.0, 9.0]]), np.array([[0.1, 9.0]]))
    np.testing.assert_array_equal(out["kappa_x1"], [[0, 220]])


def test_synthetic_table_is_physical():
    t = synthetic_table(np.linspace(0, 1.5, 4), np.linspace(0.4, 1.6, 4))
    assert np.all(t.table[..., :2] == 1.0)
    assert np.all(t.table[..., 2:] >= 0)
    # more attenuation -> stronger relaxation at the same exponent
    assert t.table[3, 2, 2] + t.table[3, 2, 6] > t.table[1, 2, 2] + t.table[1, 2, 6]
