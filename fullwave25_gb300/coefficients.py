"""Finite-difference coefficient tables consumed by the FDTD engine (``d``, ``dmap``, ``dcmap``).

The engine's spatial derivative is a staggered time-space stencil with eight axial taps per side
and one off-axis tap. The tap values depend on the local Courant number ``r = c*dT/dX`` through
degree-7 polynomials; there is one polynomial set for 2D and one for 3D. These polynomial
coefficients define the numerical scheme, so they must equal the reference's values bit for bit
(fullwave/solver/input_file_writer.py:183-367 for ``d``, :369-556 for ``dmap``, :558-559 for
``dcmap``, :808-821 for ``ndmap`` and the 0-based ``dcmap`` written to disk).

Table layout (both ``d`` and ``dmap``): row ``m`` in 1..8, column 0 is the axial tap applied to
the pair of samples ``(m - 1/2)`` cells either side of the staggered output point; row 1,
column 1 is the off-axis tap applied to the nearest pair shifted by one cell in each transverse
direction. All other entries are zero. The consistency condition of a first-derivative stencil,
``sum_m (2m-1) d[m,0] + 2*(ndim-1)*d[1,1] = 1``, holds for both tables to about 1e-5; the tests
check it and it is how the off-axis geometry is pinned.
"""

from __future__ import annotations

import numpy as np

# Polynomial coefficients, highest power first (r^7 ... r^0), for taps d[1..8, 0] and d[1, 1].
# 2D table: input_file_writer.py:278-366 (d) and :465-555 (dmap).
_POLY_2D = np.array(
    [
        [-0.000874634088067635, -0.00180530560296097, -0.000440512972481673,
         0.00474018847663366, -1.93097802254349e-05, -0.292328221171893,
         -6.58101498708345e-08, 1.25420636437969],
        [0.000793317828964018, 0.00161433256585486, 0.000397244786277123,
         0.00546057645976549, 1.73781972873916e-05, 0.0588754971188371,
         5.91706982879834e-08, -0.123406473759703],
        [-0.000650217700538851, -0.00116449260340413, -0.000324403734066325,
         -0.00911483710059994, -1.417399823126e-05, 0.0233184077551615,
         -4.82326094707544e-08, 0.0346342451534453],
        [0.000467529510541428, 0.000732736676632388, 0.000232444388955328,
         0.00846419766685254, 1.01438593426278e-05, -0.0317586249260511,
         3.44988852042879e-08, -0.0119674942518101],
        [-0.000298416281187033, -0.000399380750669364, -0.000148203388388213,
         -0.00601788793192501, -6.46543538517443e-06, 0.0241912754935119,
         -2.19855171569984e-08, 0.00415554391204146],
        [0.000167882669698981, 0.000188195874702691, 8.3057921860396e-05,
         0.00348461963201376, 3.61873162287129e-06, -0.0149875789940005,
         1.22979142197165e-08, -0.00129213888778954],
        [-6.22209937489143e-05, -6.44890425871692e-05, -3.02936928954918e-05,
         -0.00133386143898282, -1.31215186728213e-06, 0.00670228205200379,
         -4.44653967516776e-09, 0.000315659916047599],
        [6.8474088109024e-06, 1.14082245705934e-05, 3.0372759370575e-06,
         0.000236122782444105, 1.26768491232397e-07, -0.00153347270556276,
         4.21617557752767e-10, -4.51948990428065e-05],
        # off-axis tap d[1, 1]
        [2.13188763071246e-06, -7.41025068776257e-05, 2.31652037371554e-06,
         -0.00259495924602038, 1.20637183170338e-07, 0.0521123771632193,
         4.42258843694177e-10, -4.20967682664542e-07],
    ],
    dtype=np.float64,
)

# 3D table: input_file_writer.py:187-276 (d) and :372-463 (dmap).
_POLY_3D = np.array(
    [
        [3.26627215252963e-3, -7.91679373564790e-4, 1.08663532410570e-3,
         2.54974226454794e-2, 3.23083288193913e-5, -3.97704676886853e-1,
         7.95584310128586e-8, 1.25425295688331],
        [-2.83291379048757e-3, 8.52796449228369e-4, -9.45353822586534e-4,
         -8.82015372858580e-3, -2.81364895458027e-5, 6.73021045987599e-2,
         -6.93180036837075e-8, -1.23448809066664e-1],
        [2.32775473203342e-3, -5.56793042789852e-4, 7.77649035879584e-4,
         2.45547234243566e-3, 2.31537892801923e-5, 1.61900960524164e-2,
         5.70523152308121e-8, 3.46683979649506e-2],
        [-1.68883462553539e-3, 3.03535823592644e-4, -5.64777117315819e-4,
         2.44582905523866e-4, -1.68215579314751e-5, -2.62344345204941e-2,
         -4.14559953526389e-8, -1.19918511290930e-2],
        [1.08994931098070e-3, -1.41445142143525e-4, 3.64794490139160e-4,
         -8.86057426195227e-4, 1.08681882832738e-5, 2.07238558666603e-2,
         2.67876079477806e-8, 4.17058420250698e-3],
        [-6.39950124405340e-4, 6.06079815415080e-5, -2.14633466007892e-4,
         6.84580412267934e-4, -6.39907927898092e-6, -1.29825288653404e-2,
         -1.57775422151124e-8, -1.29998325971518e-3],
        [2.92716539609611e-4, -1.87446062803024e-5, 9.85389372183761e-5,
         -2.40360290348543e-4, 2.94166215515130e-6, 5.57066438452790e-3,
         7.25741366376659e-9, 3.18698432679400e-4],
        [-6.42183857909518e-5, 3.38552867751042e-6, -2.17377151411164e-5,
         4.98269067389945e-5, -6.50197868987757e-7, -1.19096089679178e-3,
         -1.60559948991172e-9, -4.57795411807702e-5],
        # off-axis tap d[1, 1]
        [-4.47723278782936e-5, -7.69502473399932e-5, -1.41765498250133e-5,
         -2.54672045901272e-3, -4.14343385915353e-7, 5.00210047924752e-2,
         -1.01220354410507e-9, -8.07139347787336e-8],
    ],
    dtype=np.float64,
)

N_TAPS = 8  # axial taps per side; the ghost layer around the grid is this many cells


def matlab_round(value):
    """Round half away from zero like MATLAB, as ``fullwave/utils/numerical.py:22-24`` does."""
    return np.round(np.asarray(value) + 1e-9).astype(int)


def _eval_row(row: np.ndarray, r) -> float:
    # Sum of c_k * r**k, highest power first: the same operation order as the reference, so the
    # float64 result (and hence the float32 file value) is identical.
    total = row[0] * r**7
    for k, coef in enumerate(row[1:], start=1):
        power = 7 - k
        if power >= 2:
            total = total + coef * r**power
        elif power == 1:
            total = total + coef * r
        else:
            total = total + coef
    return total


def _table(is_3d: bool) -> np.ndarray:
    return _POLY_3D if is_3d else _POLY_2D


def d_matrix(cfl: float, *, is_3d: bool) -> np.ndarray:
    """Return the global ``d`` table, shape ``[9, 2]`` float64, evaluated at ``r = cfl``."""
    poly = _table(is_3d)
    d = np.zeros((9, 2))
    for m in range(1, 9):
        d[m, 0] = _eval_row(poly[m - 1], cfl)
    d[1, 1] = _eval_row(poly[8], cfl)
    return d


def d_map(sound_speed: np.ndarray, dt: float, dx: float, *, is_3d: bool) -> np.ndarray:
    """Return ``dmap``, shape ``[9, 2, ndim_c + 1]`` float64, one tap set per integer sound speed.

    Entry ``i`` is evaluated at ``r = (c_min + i) * dt / dx``; the number of entries is
    ``round(c_max) - round(c_min) + 1`` (input_file_writer.py:95-101, :369-372).
    """
    c = np.asarray(sound_speed)
    span = int(matlab_round(c.max()) - matlab_round(c.min()))
    cmin = c.min()
    poly = _table(is_3d)
    out = np.zeros((9, 2, span + 1))
    for i in range(span + 1):
        r = (i + cmin) * dt / dx
        for m in range(1, 9):
            out[m, 0, i] = _eval_row(poly[m - 1], r)
        out[1, 1, i] = _eval_row(poly[8], r)
    return out


def dc_map(sound_speed: np.ndarray) -> np.ndarray:
    """Return the 0-based per-cell tap-set index ``round(c) - round(c_min)`` (int32)."""
    c = np.asarray(sound_speed)
    return (matlab_round(c) - matlab_round(c.min())).astype(np.int32)


def n_dmap(dmap: np.ndarray) -> int:
    """Number of tap sets the engine reads; 1 for a homogeneous medium (input_file_writer.py:808-811)."""
    return 1 if dmap.shape[2] == 1 else int(dmap.shape[2])


def consistency_residual(d: np.ndarray, *, is_3d: bool) -> float:
    """``sum_m (2m-1) d[m,0] + 2*(ndim-1) d[1,1] - 1`` for a tap table (zero for a consistent stencil)."""
    n_offaxis_pairs = 4 if is_3d else 2
    m = np.arange(1, 9)
    return float(((2 * m - 1) * d[1:9, 0]).sum() + n_offaxis_pairs * d[1, 1] - 1.0)


def pack_taps(dmap: np.ndarray) -> np.ndarray:
    """Pack ``dmap[9,2,n]`` into the engine's device table ``[n, 12]`` float32.

    Columns 0..7 hold the axial taps ``d[1..8, 0]``, column 8 the off-axis tap ``d[1, 1]`` and
    columns 9..11 are zero padding so that each tap set is three 16-byte vectors.
    """
    n = dmap.shape[2]
    out = np.zeros((n, 12), dtype=np.float32)
    out[:, 0:8] = dmap[1:9, 0, :].T.astype(np.float32)
    out[:, 8] = dmap[1, 1, :].astype(np.float32)
    return out
