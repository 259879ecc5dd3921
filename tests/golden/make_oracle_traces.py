"""Record the FP64 oracle's sensor traces for the golden input sets (``oracle_traces.npz``).

    python tests/golden/make_oracle_traces.py

The CPU test suite re-runs the oracle on the same inputs and compares against these traces, so
any change to the oracle's arithmetic shows up as a test failure.
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path[:0] = [str(HERE.parent.parent), str(HERE.parent.parent / "oracle")]

from fdtd_oracle import run_oracle  # noqa: E402
from golden_io import CASE_NAMES, load_case_inputs  # noqa: E402


def main():
    out = {}
    for name in CASE_NAMES:
        out[name] = run_oracle(load_case_inputs(name))
        print(name, out[name].shape, float(np.abs(out[name]).max()))
    np.savez_compressed(HERE / "oracle_traces.npz", **out)


if __name__ == "__main__":
    main()
