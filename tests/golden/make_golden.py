"""Generate the golden fixtures in this folder from the reference's own Python pre-processing.

Run where a checkout of the reference is available (it is only read):

    python tests/golden/make_golden.py --reference <reference checkout> [--only NAME,...]

(or set ``FULLWAVE_REFERENCE`` to the checkout instead of passing ``--reference``). ``--only``
regenerates a subset: ``coeff``, ``cases``, ``exp_cases``, ``pulse``, ``transducer``.

The reference imports matplotlib, cv2 and tqdm only for plotting and progress bars; this script
puts empty stand-ins for them on ``sys.path`` (in a temporary folder) before importing it. Nothing
here runs the reference's engine executables. Outputs (committed):

* ``coeff_tables.npz``: the reference's ``d`` (2D/3D at several Courant numbers) and ``dmap`` /
  ``dcmap`` tables (``InputFileWriter._set_d_mat`` / ``_set_d_map`` / ``_set_dc_map``).
* ``case_<name>.npz``: the complete ``.dat`` input set that ``PMLBuilder.run`` +
  ``InputFileWriter.run`` write for a small simulation (raw file bytes per file name), plus the
  scenario that produced it (maps before PML padding, source signal and masks), so the tests can
  rebuild the same set with this repository's host builders and compare bytes.
"""

from __future__ import annotations

import argparse
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

REFERENCE: Path | None = None   # set from --reference / FULLWAVE_REFERENCE by main()
HERE = Path(__file__).resolve().parent

_STUB = '''
class _M(type):
    def __getattr__(cls, k): return _A
    def __or__(cls, o): return cls
    def __ror__(cls, o): return cls
class _A(metaclass=_M):
    def __init__(self, *a, **k): pass
    def __getattr__(self, k): return _A()
    def __call__(self, *a, **k): return _A()
    def __iter__(self): return iter([])
def __getattr__(k): return _A
'''


def _import_reference(tmp: Path):
    for pkg, subs in (("matplotlib", ("pyplot", "axes", "figure", "colors", "patches",
                                      "animation", "cm")), ("cv2", ())):
        (tmp / pkg).mkdir()
        (tmp / pkg / "__init__.py").write_text(_STUB)
        for s in subs:
            (tmp / pkg / f"{s}.py").write_text(_STUB)
    (tmp / "tqdm").mkdir()
    (tmp / "tqdm" / "__init__.py").write_text("def tqdm(it=None, *a, **k):\n    return it\n")
    sys.path[:0] = [str(tmp), str(REFERENCE)]
    import fullwave  # noqa: PLC0415
    return fullwave


def relaxation_maps(rng, shape, scale=1.0):
    """Plausible two-mechanism relaxation maps (kappa ~ 1, d ~ 1e4..1e5 /s, alpha ~ 1e6..1e8 /s)."""
    lo = lambda a, b: rng.uniform(a, b, size=shape)  # noqa: E731
    return {
        "kappa_x1": lo(1.0, 1.004), "kappa_x2": lo(1.0, 1.004),
        "d_x1_nu1": scale * lo(1e4, 6e4), "alpha_x1_nu1": lo(5e6, 2e7),
        "d_x2_nu1": scale * lo(1e4, 6e4), "alpha_x2_nu1": lo(5e6, 2e7),
        "d_x1_nu2": scale * lo(2e4, 9e4), "alpha_x1_nu2": lo(3e7, 1.2e8),
        "d_x2_nu2": scale * lo(2e4, 9e4), "alpha_x2_nu2": lo(3e7, 1.2e8),
    }


def smooth(rng, shape, lo, hi, blobs=3):
    """Background plus a few rectangular inclusions: a heterogeneous but simple map."""
    out = np.full(shape, (lo + hi) / 2.0)
    for _ in range(blobs):
        sl = tuple(slice(int(a), int(a) + max(2, int(n) // 3))
                   for a, n in zip(rng.integers(0, np.array(shape) // 2), shape))
        out[sl] = rng.uniform(lo, hi)
    return out


CASES = {
    # name: (shape, f0, nt, ppw, cfl, n_pml, n_transition, mod_t, beta, air, use_pml, src_layers
    #        [, isotropic])
    "2d_small": ((40, 36), 3e6, 240, 12, 0.2, 6, 6, 1, 0.0, False, True, 3),
    "2d_air_beta": ((36, 32), 3e6, 200, 12, 0.25, 5, 5, 3, 3.5, True, True, 2),
    "2d_nopml": ((30, 28), 2e6, 150, 10, 0.3, 0, 0, 2, 0.0, False, False, 1),
    "3d_small": ((16, 14, 12), 2e6, 120, 10, 0.2, 3, 3, 2, 0.0, False, True, 2),
    "2d_aniso": ((34, 30), 3e6, 160, 12, 0.2, 5, 5, 1, 0.0, False, True, 2, False),
    "3d_aniso": ((14, 12, 12), 2e6, 90, 10, 0.2, 3, 3, 1, 0.0, False, True, 1, False),
}


def build_case(fw, name, spec, tmp: Path):
    shape, f0, nt, ppw, cfl, n_pml, n_tr, mod_t, beta, air, use_pml, layers = spec[:12]
    iso = spec[12] if len(spec) > 12 else True
    rng = np.random.default_rng(sum(map(ord, name)))
    c0 = 1540.0
    dx = c0 / f0 / ppw
    dt = cfl * dx / c0
    grid = fw.Grid(domain_size=tuple(n * dx for n in shape), f0=f0, duration=nt * dt, c0=c0,
                   ppw=ppw, cfl=cfl)
    assert grid.shape == shape and grid.nt == nt, (grid.shape, grid.nt)
    c = smooth(rng, shape, 1480.0, 1620.0)
    rho = smooth(rng, shape, 950.0, 1080.0)
    beta_map = np.full(shape, beta)
    air_map = np.zeros(shape, dtype=bool)
    if air:
        air_map[tuple(slice(n - 6, n - 2) for n in shape)] = True
    relax = relaxation_maps(rng, shape)
    medium = fw.MediumRelaxationMaps(grid, c, rho, beta_map, relax, air_map=air_map,
                                     use_isotropic_relaxation=iso)
    src_mask = np.zeros(shape, dtype=bool)
    src_mask[:layers] = True
    coords = np.array(np.where(src_mask)).T
    per_layer = coords.shape[0] // layers
    p0 = np.zeros((coords.shape[0], nt))
    for i in range(layers):
        p0[i * per_layer:(i + 1) * per_layer] = fw.utils.pulse.gaussian_modulated_sinusoidal_signal(
            nt=nt, duration=grid.duration, ncycles=2, drop_off=2, f0=f0, p0=1e5, i_layer=i,
            dt_for_layer_delay=grid.dt, cfl_for_layer_delay=grid.cfl)
    source = fw.Source(p0, src_mask)
    sens_mask = np.zeros(shape, dtype=bool)
    sens_mask[min(layers + 4, shape[0] - 1)] = True
    sens_mask[shape[0] // 2, shape[1] // 3] = True
    sens_mask[-3, 2] = True
    sensor = fw.Sensor(sens_mask, sampling_modulus_time=mod_t)

    from fullwave.solver.input_file_writer import InputFileWriter  # noqa: PLC0415
    from fullwave.solver.pml_builder import PMLBuilder  # noqa: PLC0415

    builder = PMLBuilder(grid, medium, source, sensor, m_spatial_order=8, n_pml_layer=n_pml,
                         n_transition_layer=n_tr, use_isotropic_relaxation=iso)
    ext_medium = builder.run(use_pml=use_pml)
    dummy_bin = tmp / "engine_placeholder"
    dummy_bin.write_text("placeholder: the engine executable is not copied into fixtures\n")
    writer = InputFileWriter(work_dir=tmp / "work", grid=builder.extended_grid,
                             medium=ext_medium, source=builder.extended_source,
                             sensor=builder.extended_sensor, path_fullwave_simulation_bin=dummy_bin,
                             use_isotropic_relaxation=iso)
    sim_dir = writer.run(name)
    files = {f"dat/{p.stem}": np.frombuffer(p.read_bytes(), dtype=np.uint8)
             for p in sorted(sim_dir.glob("*.dat"))}
    scenario = {"shape": np.array(shape), "f0": f0, "nt": nt, "ppw": ppw, "cfl": cfl,
                "n_pml": n_pml, "n_transition": n_tr, "mod_t": mod_t, "use_pml": use_pml,
                "isotropic": iso,
                "c": c, "rho": rho, "beta": beta_map, "air_map": air_map, "p0": p0,
                "src_mask": src_mask, "sens_mask": sens_mask,
                **{f"relax/{k}": v for k, v in relax.items()}}
    np.savez_compressed(HERE / f"case_{name}.npz", **files, **scenario)
    print(f"case {name}: extended grid {builder.extended_grid.shape}, {len(files)} files")


EXP_CASES = {
    # name: (shape, f0, nt, ppw, cfl, n_pml, mod_t, use_pml)
    "2d_exp": ((36, 30), 3e6, 160, 12, 0.2, 8, 1, True),
    "3d_exp": ((14, 12, 12), 2e6, 90, 10, 0.2, 4, 2, True),
}


def build_exp_case(fw, name, spec, tmp: Path):
    """Exponential-attenuation input set (PMLBuilderExponentialAttenuation + InputFileWriter
    with use_exponential_attenuation=True). The relaxation lookup table is not read on this
    path; Medium only checks that its file exists, so an empty placeholder is passed."""
    shape, f0, nt, ppw, cfl, n_pml, mod_t, use_pml = spec
    rng = np.random.default_rng(sum(map(ord, name)))
    c0 = 1540.0
    dx = c0 / f0 / ppw
    dt = cfl * dx / c0
    grid = fw.Grid(domain_size=tuple(n * dx for n in shape), f0=f0, duration=nt * dt, c0=c0,
                   ppw=ppw, cfl=cfl)
    c = smooth(rng, shape, 1480.0, 1620.0)
    rho = smooth(rng, shape, 950.0, 1080.0)
    a0 = smooth(rng, shape, 0.2, 1.2)
    placeholder = tmp / "lut_placeholder.mat"
    placeholder.write_bytes(b"")
    medium = fw.Medium(grid, c, rho, a0, np.full(shape, 1.1), np.zeros(shape),
                       path_relaxation_parameters_database=placeholder)
    src_mask = np.zeros(shape, dtype=bool)
    src_mask[0] = True
    n_src = int(src_mask.sum())
    p0 = np.tile(fw.utils.pulse.gaussian_modulated_sinusoidal_signal(
        nt=nt, duration=grid.duration, ncycles=2, drop_off=2, f0=f0, p0=1e5), (n_src, 1))
    source = fw.Source(p0, src_mask)
    sens_mask = np.zeros(shape, dtype=bool)
    sens_mask[4] = True
    sensor = fw.Sensor(sens_mask, sampling_modulus_time=mod_t)

    from fullwave.solver.input_file_writer import InputFileWriter  # noqa: PLC0415
    from fullwave.solver.pml_builder import PMLBuilderExponentialAttenuation  # noqa: PLC0415

    builder = PMLBuilderExponentialAttenuation(grid, medium, source, sensor, m_spatial_order=8,
                                               n_pml_layer=n_pml)
    ext_medium = builder.run(use_pml=use_pml)
    dummy_bin = tmp / "engine_placeholder"
    dummy_bin.write_text("placeholder\n")
    writer = InputFileWriter(work_dir=tmp / "work", grid=builder.extended_grid,
                             medium=ext_medium, source=builder.extended_source,
                             sensor=builder.extended_sensor, path_fullwave_simulation_bin=dummy_bin,
                             use_exponential_attenuation=True)
    sim_dir = writer.run(name)
    files = {f"dat/{p.stem}": np.frombuffer(p.read_bytes(), dtype=np.uint8)
             for p in sorted(sim_dir.glob("*.dat"))}
    scenario = {"shape": np.array(shape), "f0": f0, "nt": nt, "ppw": ppw, "cfl": cfl,
                "n_pml": n_pml, "mod_t": mod_t, "use_pml": use_pml, "c": c, "rho": rho,
                "alpha_coeff": a0, "p0": p0, "src_mask": src_mask, "sens_mask": sens_mask}
    np.savez_compressed(HERE / f"case_{name}.npz", **files, **scenario)
    print(f"exp case {name}: extended grid {builder.extended_grid.shape}, {len(files)} files")


def coefficient_tables(fw, tmp: Path):
    from fullwave.solver.input_file_writer import InputFileWriter  # noqa: PLC0415

    out = {}
    for is_3d in (False, True):
        for cfl in (0.05, 0.1, 0.2, 0.3, 0.45):
            w = object.__new__(InputFileWriter)
            w.is_3d = is_3d
            w.grid = type("G", (), {"cfl": cfl})()
            w._set_d_mat()
            out[f"d_{'3d' if is_3d else '2d'}_cfl{cfl}"] = w._d
        dx = 1540 / 3e6 / 12
        dt = 0.2 * dx / 1540
        c = np.linspace(1450.3, 1650.7, 97)
        w = object.__new__(InputFileWriter)
        w.is_3d = is_3d
        w.grid = type("G", (), {"dt": dt, "dx": dx})()
        dim = int(np.round(c.max() + 1e-9) - np.round(c.min() + 1e-9))
        w._set_d_map(dim, c)
        w._set_dc_map(c)
        tag = "3d" if is_3d else "2d"
        out[f"dmap_{tag}"] = w._d_map
        out[f"dcmap_{tag}"] = w._dc_map - 1
        out[f"dmap_c_{tag}"] = c
        out[f"dmap_dt_{tag}"] = dt
        out[f"dmap_dx_{tag}"] = dx
    np.savez_compressed(HERE / "coeff_tables.npz", **out)
    print(f"coeff_tables: {len(out)} arrays")


PULSE_PARAMS = [
    # nt, duration factor (x nt dt), ncycles, drop_off, f0, p0, delay_sec, i_layer
    (400, 1.0, 2, 2, 3e6, 1e6, 0.0, 0),
    (600, 1.0, 3, 1, 2.5e6, 2e5, 1.5e-7, 0),
    (500, 1.0, 2, 2, 5e6, 1e6, 0.0, 3),
    (300, 1.0, 1, 3, 4e6, 1.0, -2e-8, 1),
]


def pulse_golden(fw):
    from fullwave.utils.pulse import gaussian_modulated_sinusoidal_signal  # noqa: PLC0415

    out = {}
    for k, (nt, fac, ncyc, drop, f0, p0, delay, layer) in enumerate(PULSE_PARAMS):
        dx = 1540.0 / f0 / 12
        dt = 0.2 * dx / 1540.0
        kw = dict(nt=nt, duration=fac * nt * dt, ncycles=ncyc, drop_off=drop, f0=f0, p0=p0,
                  delay_sec=delay)
        if layer:
            kw.update(i_layer=layer, dt_for_layer_delay=dt, cfl_for_layer_delay=0.2)
        out[f"signal_{k}"] = gaussian_modulated_sinusoidal_signal(**kw)
        out[f"params_{k}"] = np.array([nt, fac * nt * dt, ncyc, drop, f0, p0, delay, layer, dt, 0.2])
    np.savez_compressed(HERE / "pulse.npz", **out)
    print(f"pulse: {len(PULSE_PARAMS)} signals")


def transducer_golden(fw):
    from fullwave.transducer import Transducer, TransducerGeometry  # noqa: PLC0415

    f0, c0, ppw, cfl, nt = 3e6, 1540.0, 12, 0.2, 60
    dx = c0 / f0 / ppw
    out = {}
    layouts = {
        "linear": ((40, 60), dict(number_elements=8, element_width_px=4, element_spacing_px=2,
                                  element_layer_px=2, position_px=(3, 5)),
                   (True, False, True, True, True, False, True, True)),
        # with this pixel layout the convex array's element 7 has no sensor on its surface (the
        # reference's own geometry), so it is inactive here, like element 3
        "convex": ((80, 120), dict(number_elements=12, element_width_px=5, element_spacing_px=1,
                                   element_layer_px=2, position_px=(6, 20), radius=0.1),
                   (True, True, False, True, True, True, False, True, True, True, True, True)),
    }
    rng = np.random.default_rng(7)
    for name, (shape, geo, active) in layouts.items():
        grid = fw.Grid(domain_size=(shape[0] * dx, shape[1] * dx), f0=f0,
                       duration=nt * cfl * dx / c0, c0=c0, ppw=ppw, cfl=cfl)
        geom = TransducerGeometry(grid, **geo)
        tr = Transducer(geom, grid, active_sensor_elements=active)
        oc = np.asarray(tr.sensor.outcoords)
        surf = tr.element_id_to_element_surface
        ids = np.concatenate([np.full(len(v), k) for k, v in sorted(surf.items())])
        coords = np.concatenate([np.asarray(v).reshape(-1, 2) for _, v in sorted(surf.items())])
        traces = rng.standard_normal((oc.shape[0], nt)).astype(np.float32)
        out[f"{name}/outcoords"] = oc
        out[f"{name}/surface_id"] = ids
        out[f"{name}/surface_coords"] = coords
        out[f"{name}/active"] = np.asarray(tr.active_sensor_elements, dtype=bool)
        out[f"{name}/traces"] = traces
        out[f"{name}/averaged"] = tr.post_process_sensor_output(traces)
        out[f"{name}/centre"] = tr.post_process_sensor_output(traces,
                                                              average_surface_signals=False)
        print(f"transducer {name}: {oc.shape[0]} sensors, {int(out[f'{name}/active'].sum())} "
              "active elements")
    np.savez_compressed(HERE / "transducer_post.npz", **out)


def main():
    global REFERENCE
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", default=os.environ.get("FULLWAVE_REFERENCE"),
                    help="checkout of the reference package (or FULLWAVE_REFERENCE)")
    ap.add_argument("--only", default="coeff,cases,exp_cases,pulse,transducer")
    args = ap.parse_args()
    if not args.reference:
        ap.error("pass --reference <checkout> or set FULLWAVE_REFERENCE")
    REFERENCE = Path(args.reference)
    only = set(args.only.split(","))
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)
        stub_dir = tmp / "stubs"
        stub_dir.mkdir()
        fw = _import_reference(stub_dir)
        if "coeff" in only:
            coefficient_tables(fw, tmp)
        if "cases" in only:
            for name, spec in CASES.items():
                build_case(fw, name, spec, tmp)
        if "exp_cases" in only:
            for name, spec in EXP_CASES.items():
                build_exp_case(fw, name, spec, tmp)
        if "pulse" in only:
            pulse_golden(fw)
        if "transducer" in only:
            transducer_golden(fw)


if __name__ == "__main__":
    main()
