"""The C oracle is a second restatement of the NumPy oracle: identical FP64 results."""

import numpy as np
import pytest

from fdtd_oracle import run_oracle
from fdtd_oracle_c import run_oracle_c
from golden_io import CASE_NAMES, HERE, load_case_inputs

TRACES = np.load(HERE / "oracle_traces.npz")


@pytest.mark.parametrize("name", CASE_NAMES)
def test_c_oracle_equals_numpy_oracle(name):
    np.testing.assert_array_equal(run_oracle_c(load_case_inputs(name)), TRACES[name])


def test_c_oracle_workload_sample_matches_numpy():
    from fullwave25_gb300.workloads import plain_2d_inputs

    inp = plain_2d_inputs(shape=(80, 64), nt=120, n_pml=10, n_transition=10)
    np.testing.assert_array_equal(run_oracle_c(inp), run_oracle(inp))
