"""The engine's input set, built in memory or read from / written to a simulation directory.

The set of arrays and scalars is the reference engine's file contract: what
``InputFileWriter.run`` writes (fullwave/solver/input_file_writer.py:105-179, :563-827) and the
closed executable reads from its working directory. Dtypes and layouts:

* scalars ``nX nY [nZ] nT nTic modT ncoords ncoordsout ncoordszero ndmap``: int32;
  ``dX dY [dZ] dT c0``: float32 (input_file_writer.py:766-803);
* maps ``c rho K beta kappax kappau apml{u,x}{1,2} bpml{u,x}{1,2}``: float32, C order
  ``[nX, nY(, nZ)]`` (:716-751, :870-881);
* ``d`` float32 ``[9, 2]``, ``dmap`` float32 ``[9, 2, ndmap]``, ``dcmap`` int32 ``[nX, nY(, nZ)]``
  holding ``round(c) - round(c_min)`` (:805-821);
* ``icc``, ``outc``, ``icczero``: int32 ``[n, ndim]`` row-major ``(x, y[, z])`` (:841-859);
* ``icmat``: float32 ``[ncoords, nTic]`` source-major (:829-839);
* output ``genout.dat``: float32 ``[n_out, ncoordsout]`` time-major, read back by
  ``load_dat_data`` (fullwave/solver/utils.py:12-45).
"""

from __future__ import annotations

import logging
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import coefficients
from .coords import map_to_coords

logger = logging.getLogger("__main__." + __name__)

ISOTROPIC_MAPS = ("kappax", "kappau", "apmlu1", "bpmlu1", "apmlx1", "bpmlx1",
                  "apmlu2", "bpmlu2", "apmlx2", "bpmlx2")

# Gradient (nabla_1) maps per derivative axis x, y, z and divergence (nabla_2) maps per axis, as
# the anisotropic build reads them (input_file_writer.py:592-620): u/w/v for the pressure
# gradient along x/y/z, x/y/z for the velocity divergence along x/y/z.
GRAD_AXIS_LETTER = ("u", "w", "v")
DIV_AXIS_LETTER = ("x", "y", "z")


def axis_maps(letter: str) -> tuple:
    return (f"kappa{letter}", f"apml{letter}1", f"bpml{letter}1", f"apml{letter}2",
            f"bpml{letter}2")


def anisotropic_extra_maps(ndim: int) -> tuple:
    """Maps the anisotropic engine reads in addition to ISOTROPIC_MAPS."""
    out = []
    for a in range(1, ndim):
        out += axis_maps(GRAD_AXIS_LETTER[a]) + axis_maps(DIV_AXIS_LETTER[a])
    return tuple(out)


@dataclass
class EngineInputs:
    """Everything one forward solve reads (the isotropic two-mechanism engine)."""

    shape: tuple                 # (nX, nY) or (nX, nY, nZ)
    nt: int
    spacing: tuple               # (dX, dY[, dZ])
    dt: float
    c0: float
    mod_t: int
    d: np.ndarray                # [9, 2]
    dmap: np.ndarray             # [9, 2, ndmap]
    dcmap: np.ndarray            # int32 shape
    maps: dict                   # name -> float32 array of `shape` (c, rho, K, beta + ISOTROPIC_MAPS)
    icc: np.ndarray              # int32 [ncoords, ndim]
    icmat: np.ndarray            # float32 [ncoords, nTic]
    outc: np.ndarray             # int32 [ncoordsout, ndim]
    icczero: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))

    @property
    def ndim(self) -> int:
        return len(self.shape)

    @property
    def isotropic(self) -> bool:
        """True unless per-direction relaxation maps (kappay, apmlw1, ...) are present."""
        return "kappay" not in self.maps

    @property
    def exponential(self) -> bool:
        """The exponential-attenuation engine (map a_exp, no relaxation memory variables)."""
        return "a_exp" in self.maps

    @property
    def n_cells(self) -> int:
        return int(np.prod(self.shape))

    @property
    def nt_ic(self) -> int:
        return int(self.icmat.shape[1])

    @property
    def n_out(self) -> int:
        """Recorded time samples: steps ``n`` with ``n % modT == 0``."""
        return (self.nt + self.mod_t - 1) // self.mod_t

    @property
    def ndmap(self) -> int:
        return coefficients.n_dmap(self.dmap)

    def validate(self) -> None:
        """Shape and range checks; raises ``ValueError`` with the offending item."""
        if self.ndim not in (2, 3):
            raise ValueError(f"grid must be 2D or 3D, got shape {self.shape}")
        if min(self.shape) < 2 * coefficients.N_TAPS + 1:
            raise ValueError(f"every axis needs more than {2 * coefficients.N_TAPS} cells: {self.shape}")
        if self.nt < 0 or self.mod_t < 1:
            raise ValueError(f"bad nT={self.nt} or modT={self.mod_t}")
        names = ("c", "rho", "K", "beta", *ISOTROPIC_MAPS)
        if not self.isotropic:
            names += anisotropic_extra_maps(self.ndim)
        if self.exponential:
            names = ("c", "rho", "K", "beta", "a_exp")
        for name in names:
            if name not in self.maps:
                raise ValueError(f"missing map {name}")
            if tuple(self.maps[name].shape) != tuple(self.shape):
                raise ValueError(f"map {name} has shape {self.maps[name].shape}, grid is {self.shape}")
        if tuple(self.dcmap.shape) != tuple(self.shape):
            raise ValueError("dcmap shape differs from the grid")
        if self.dcmap.size and (self.dcmap.min() < 0 or self.dcmap.max() >= self.dmap.shape[2]):
            raise ValueError("dcmap indexes outside dmap")
        for name, coords in (("icc", self.icc), ("outc", self.outc), ("icczero", self.icczero)):
            if coords.size and (coords.ndim != 2 or coords.shape[1] != self.ndim):
                raise ValueError(f"{name} must be [n, {self.ndim}]")
            if coords.size and ((coords < 0).any() or (coords >= np.array(self.shape)).any()):
                raise ValueError(f"{name} has coordinates outside the grid")
        if self.icmat.shape[0] != self.icc.shape[0]:
            raise ValueError("icmat rows differ from the number of source coordinates")


def build_inputs(grid, medium, source, sensor) -> EngineInputs:
    """In-memory equivalent of ``InputFileWriter(...).run`` for the isotropic engine.

    ``grid``/``medium``/``source``/``sensor`` are the extended (PML-padded) objects, as
    ``Solver.run`` passes them to the writer (fullwave/solver/solver.py:733-745).
    """
    c = medium.sound_speed
    d = coefficients.d_matrix(grid.cfl, is_3d=grid.is_3d)
    dmap = coefficients.d_map(c, grid.dt, grid.dx, is_3d=grid.is_3d)
    fw2 = medium.relaxation_param_dict_for_fw2
    letters = ["u", "x"]
    if "kappa_y" in fw2:  # anisotropic: one set of maps per derivative direction
        nd = 3 if grid.is_3d else 2
        letters = list(GRAD_AXIS_LETTER[:nd]) + list(DIV_AXIS_LETTER[:nd])
    names = {}
    for ax in letters:
        names[f"kappa{ax}"] = f"kappa_{ax}"
        for nu in (1, 2):
            names[f"apml{ax}{nu}"] = f"a_pml_{ax}{nu}"
            names[f"bpml{ax}{nu}"] = f"b_pml_{ax}{nu}"
    maps = {"c": c.astype(np.float32), "rho": medium.density.astype(np.float32),
            "K": medium.bulk_modulus.astype(np.float32), "beta": medium.beta.astype(np.float32)}
    for fw_name, key in names.items():
        maps[fw_name] = np.asarray(fw2[key]).astype(np.float32)
    spacing = (grid.dx, grid.dy, grid.dz) if grid.is_3d else (grid.dx, grid.dy)
    return EngineInputs(
        shape=tuple(grid.shape), nt=int(grid.nt), spacing=spacing, dt=grid.dt, c0=grid.c0,
        mod_t=int(sensor.sampling_modulus_time), d=d, dmap=dmap,
        dcmap=coefficients.dc_map(c), maps=maps,
        icc=source.incoords.astype(np.int32), icmat=np.asarray(source.icmat, dtype=np.float32),
        outc=sensor.outcoords.astype(np.int32),
        icczero=map_to_coords(medium.air_map).astype(np.int32).reshape(-1, grid.is_3d + 2),
    )


def build_inputs_exponential(grid, medium, source, sensor) -> EngineInputs:
    """In-memory equivalent of ``InputFileWriter`` with ``use_exponential_attenuation=True``
    (input_file_writer.py:629-645): maps c, K, rho, beta, a_exp plus the shared contract."""
    c = medium.sound_speed
    maps = {"c": c.astype(np.float32), "rho": medium.density.astype(np.float32),
            "K": medium.bulk_modulus.astype(np.float32), "beta": medium.beta.astype(np.float32),
            "a_exp": medium.alpha_exp.astype(np.float32)}
    spacing = (grid.dx, grid.dy, grid.dz) if grid.is_3d else (grid.dx, grid.dy)
    return EngineInputs(
        shape=tuple(grid.shape), nt=int(grid.nt), spacing=spacing, dt=grid.dt, c0=grid.c0,
        mod_t=int(sensor.sampling_modulus_time),
        d=coefficients.d_matrix(grid.cfl, is_3d=grid.is_3d),
        dmap=coefficients.d_map(c, grid.dt, grid.dx, is_3d=grid.is_3d),
        dcmap=coefficients.dc_map(c), maps=maps,
        icc=source.incoords.astype(np.int32), icmat=np.asarray(source.icmat, dtype=np.float32),
        outc=sensor.outcoords.astype(np.int32),
        icczero=map_to_coords(medium.air_map).astype(np.int32).reshape(-1, grid.is_3d + 2),
    )


# -- simulation-directory (.dat) contract -------------------------------------------------------

def _read(path: Path, dtype, count=-1) -> np.ndarray:
    if not path.exists():
        raise ValueError(f"dat_file_path {path} does not exist")
    return np.fromfile(path, dtype=dtype, count=count)


def read_simulation_dir(sim_dir: Path) -> EngineInputs:
    """Read the engine inputs that ``InputFileWriter`` left in ``sim_dir`` (isotropic build)."""
    sim_dir = Path(sim_dir)
    i32 = lambda n: int(_read(sim_dir / f"{n}.dat", np.int32, 1)[0])  # noqa: E731
    f32 = lambda n: float(_read(sim_dir / f"{n}.dat", np.float32, 1)[0])  # noqa: E731
    is_3d = (sim_dir / "nZ.dat").exists()
    shape = (i32("nX"), i32("nY"), i32("nZ")) if is_3d else (i32("nX"), i32("nY"))
    spacing = (f32("dX"), f32("dY"), f32("dZ")) if is_3d else (f32("dX"), f32("dY"))
    ndim = len(shape)
    n_cells = int(np.prod(shape))

    def grid_map(name, dtype=np.float32):
        arr = _read(sim_dir / f"{name}.dat", dtype)
        if arr.size != n_cells:
            raise ValueError(f"{name}.dat holds {arr.size} values, grid has {n_cells}")
        return arr.reshape(shape)

    ncoords, ncoordsout, ncoordszero = i32("ncoords"), i32("ncoordsout"), i32("ncoordszero")
    nt_ic = i32("nTic")
    ndmap = i32("ndmap")
    dmap = _read(sim_dir / "dmap.dat", np.float32)
    if dmap.size % 18:
        raise ValueError("dmap.dat is not a [9, 2, n] table")
    dmap = dmap.reshape(9, 2, -1)
    if ndmap != dmap.shape[2] and not (ndmap == 1 and dmap.shape[2] >= 1):
        raise ValueError(f"ndmap={ndmap} disagrees with dmap.dat ({dmap.shape[2]} tap sets)")
    names = ("c", "rho", "K", "beta", *ISOTROPIC_MAPS)
    if (sim_dir / "kappay.dat").exists():
        names += anisotropic_extra_maps(len(shape))
    if (sim_dir / "a_exp.dat").exists() and not (sim_dir / "kappax.dat").exists():
        names = ("c", "rho", "K", "beta", "a_exp")
    maps = {n: grid_map(n) for n in names}
    coords = lambda n, k: _read(sim_dir / f"{n}.dat", np.int32).reshape(k, ndim)  # noqa: E731
    icczero = (coords("icczero", ncoordszero) if ncoordszero
               else np.zeros((0, ndim), np.int32))
    return EngineInputs(
        shape=shape, nt=i32("nT"), spacing=spacing, dt=f32("dT"), c0=f32("c0"),
        mod_t=i32("modT"), d=_read(sim_dir / "d.dat", np.float32).reshape(9, 2), dmap=dmap,
        dcmap=grid_map("dcmap", np.int32), maps=maps, icc=coords("icc", ncoords),
        icmat=_read(sim_dir / "icmat.dat", np.float32).reshape(ncoords, nt_ic),
        outc=coords("outc", ncoordsout), icczero=icczero,
    )


def write_simulation_dir(inputs: EngineInputs, sim_dir: Path) -> Path:
    """Write ``inputs`` with the same file names, dtypes and layouts as ``InputFileWriter``."""
    sim_dir = Path(sim_dir)
    sim_dir.mkdir(parents=True, exist_ok=True)
    w = lambda n, a, t: np.asarray(a).astype(t).tofile(sim_dir / f"{n}.dat")  # noqa: E731
    axes = "XYZ"[: inputs.ndim]
    for k, ax in enumerate(axes):
        w(f"n{ax}", inputs.shape[k], np.int32)
        w(f"d{ax}", inputs.spacing[k], np.float32)
    w("dT", inputs.dt, np.float32)
    w("c0", inputs.c0, np.float32)
    w("nT", inputs.nt, np.int32)
    w("ncoords", inputs.icc.shape[0], np.int32)
    w("ncoordsout", inputs.outc.shape[0], np.int32)
    w("ncoordszero", inputs.icczero.shape[0], np.int32)
    w("nTic", inputs.nt_ic, np.int32)
    w("modT", inputs.mod_t, np.int32)
    w("d", inputs.d, np.float32)
    w("dmap", inputs.dmap, np.float32)
    w("ndmap", inputs.ndmap, np.int32)
    w("dcmap", inputs.dcmap, np.int32)
    for name, arr in inputs.maps.items():
        w(name, arr, np.float32)
    w("icc", inputs.icc, np.int32)
    w("outc", inputs.outc, np.int32)
    w("icczero", inputs.icczero, np.int32)
    w("icmat", inputs.icmat, np.float32)
    return sim_dir


def load_dat_data(path: Path, dtype=np.float32) -> np.ndarray:
    """Read a flat ``.dat`` array and warn on NaN/Inf (fullwave/solver/utils.py:12-45)."""
    data = _read(Path(path), dtype)
    if np.isnan(data).any():
        logger.warning("The simulation contains NaN values. Check the simulation domains or PML settings.")
    if np.isinf(data).any():
        logger.warning("The simulation contains Inf values. Check the simulation domains or PML settings.")
    return data
