"""Helpers to read the committed golden cases (see make_golden.py for how they were made)."""

from __future__ import annotations

from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
CASE_NAMES = ("2d_small", "2d_air_beta", "2d_nopml", "3d_small", "2d_aniso", "3d_aniso",
              "2d_exp", "3d_exp")


def load_case(name: str):
    return np.load(HERE / f"case_{name}.npz")


def write_case_dir(name: str, dest: Path) -> Path:
    """Write the reference-generated ``.dat`` files of a case into ``dest``."""
    z = load_case(name)
    dest = Path(dest)
    dest.mkdir(parents=True, exist_ok=True)
    for k in z.files:
        if k.startswith("dat/"):
            (dest / f"{k[4:]}.dat").write_bytes(z[k].tobytes())
    return dest


def load_case_inputs(name: str):
    import tempfile  # noqa: PLC0415

    from fullwave25_gb300.inputs import read_simulation_dir  # noqa: PLC0415

    with tempfile.TemporaryDirectory() as td:
        return read_simulation_dir(write_case_dir(name, Path(td)))


def rebuild_case_inputs(name: str):
    """Rebuild the case's engine inputs with this repository's host builders."""
    from fullwave25_gb300.grid import Grid  # noqa: PLC0415
    from fullwave25_gb300.inputs import build_inputs  # noqa: PLC0415
    from fullwave25_gb300.medium import MediumRelaxationMaps  # noqa: PLC0415
    from fullwave25_gb300.pml import PMLBuilder  # noqa: PLC0415
    from fullwave25_gb300.source import Sensor, Source  # noqa: PLC0415

    z = load_case(name)
    shape = tuple(int(v) for v in z["shape"])
    g = Grid.from_cells(shape, f0=float(z["f0"]), nt=int(z["nt"]), ppw=int(z["ppw"]),
                        cfl=float(z["cfl"]))
    if "alpha_coeff" in z.files:  # exponential-attenuation case
        from fullwave25_gb300.exponential import PMLBuilderExponentialAttenuation  # noqa: PLC0415
        from fullwave25_gb300.inputs import build_inputs_exponential  # noqa: PLC0415

        b = PMLBuilderExponentialAttenuation(
            g, z["c"], z["rho"], z["alpha_coeff"], np.zeros(shape), Source(z["p0"], z["src_mask"]),
            Sensor(z["sens_mask"], int(z["mod_t"])), n_pml_layer=int(z["n_pml"]))
        m = b.run(use_pml=bool(z["use_pml"]))
        return build_inputs_exponential(b.extended_grid, m, b.extended_source, b.extended_sensor)
    relax = {k[6:]: z[k] for k in z.files if k.startswith("relax/")}
    iso = bool(z["isotropic"]) if "isotropic" in z.files else True
    med = MediumRelaxationMaps(g, z["c"], z["rho"], z["beta"], relax, air_map=z["air_map"],
                               use_isotropic_relaxation=iso)
    src = Source(z["p0"], z["src_mask"])
    sen = Sensor(z["sens_mask"], int(z["mod_t"]))
    b = PMLBuilder(g, med, src, sen, n_pml_layer=int(z["n_pml"]),
                   n_transition_layer=int(z["n_transition"]), use_isotropic_relaxation=iso)
    em = b.run(use_pml=bool(z["use_pml"]))
    return build_inputs(b.extended_grid, em, b.extended_source, b.extended_sensor)
