"""GPU-side pre-processing of the Solver path (``device_build.device_inputs``), run here with
torch on the CPU: the engine inputs it builds equal the reference's own ``.dat`` output for the
golden cases (every relaxation and exponential case, element by element), and equal this
package's host builders for a medium given by attenuation maps (relaxation table lookup) and for
whole-domain recording."""

import numpy as np
import pytest

from golden_io import CASE_NAMES, load_case, load_case_inputs

torch = pytest.importorskip("torch")
CPU = torch.device("cpu")


def _scenario(name):
    from fullwave25_gb300.grid import Grid
    from fullwave25_gb300.medium import Medium, MediumRelaxationMaps
    from fullwave25_gb300.source import Sensor, Source

    z = load_case(name)
    shape = tuple(int(v) for v in z["shape"])
    g = Grid.from_cells(shape, f0=float(z["f0"]), nt=int(z["nt"]), ppw=int(z["ppw"]),
                        cfl=float(z["cfl"]))
    src = Source(z["p0"], z["src_mask"])
    sen = Sensor(z["sens_mask"], int(z["mod_t"]))
    if "alpha_coeff" in z.files:
        med = Medium(g, z["c"], z["rho"], z["alpha_coeff"], np.full(shape, 1.1), np.zeros(shape))
        kw = dict(n_pml=int(z["n_pml"]), n_transition=0, use_pml=bool(z["use_pml"]),
                  use_exponential_attenuation=True)
    else:
        relax = {k[6:]: z[k] for k in z.files if k.startswith("relax/")}
        iso = bool(z["isotropic"]) if "isotropic" in z.files else True
        med = MediumRelaxationMaps(g, z["c"], z["rho"], z["beta"], relax, air_map=z["air_map"],
                                   use_isotropic_relaxation=iso)
        kw = dict(n_pml=int(z["n_pml"]), n_transition=int(z["n_transition"]),
                  use_pml=bool(z["use_pml"]), use_isotropic_relaxation=iso)
    return g, med, src, sen, kw


def _assert_equal_inputs(dev, ref):
    from fullwave25_gb300.workloads3d import to_host_inputs

    got = to_host_inputs(dev)
    assert tuple(got.shape) == tuple(ref.shape) and got.nt == ref.nt and got.mod_t == ref.mod_t
    assert np.float32(got.dt) == np.float32(ref.dt)
    assert [np.float32(s) for s in got.spacing] == [np.float32(s) for s in ref.spacing]
    assert set(got.maps) == set(ref.maps), set(got.maps) ^ set(ref.maps)
    for k in ref.maps:
        np.testing.assert_array_equal(got.maps[k], ref.maps[k], err_msg=k)
    for k in ("dcmap", "icc", "outc", "icczero", "icmat"):
        np.testing.assert_array_equal(getattr(got, k), getattr(ref, k), err_msg=k)
    np.testing.assert_array_equal(np.asarray(got.dmap, np.float32), np.asarray(ref.dmap, np.float32))
    np.testing.assert_array_equal(np.asarray(got.d, np.float32), np.asarray(ref.d, np.float32))


@pytest.mark.parametrize("name", CASE_NAMES)
def test_device_inputs_equal_reference_dat_files(name):
    from fullwave25_gb300.device_build import device_inputs

    g, med, src, sen, kw = _scenario(name)
    dev, n_sensors = device_inputs(g, med, src, sen, device=CPU, **kw)
    ref = load_case_inputs(name)
    assert n_sensors == ref.outc.shape[0]
    _assert_equal_inputs(dev, ref)


@pytest.mark.parametrize("iso", [True, False])
def test_device_inputs_from_attenuation_maps_equal_host_solver(iso):
    """A Medium (alpha0, gamma maps) through the relaxation table lookup, sort and PML."""
    from fullwave25_gb300.solver import Solver
    from fullwave25_gb300.workloads import plain_2d_problem

    grid, medium, source, sensor, _ = plain_2d_problem(shape=(90, 70), nt=120, seed=4)
    s = Solver("/tmp", grid, medium, source, sensor, pml_layer_thickness_px=10,
               n_transition_layer=12, use_isotropic_relaxation=iso)
    host, _ = s.build_engine_inputs()
    dev, n = s.build_device_inputs(device=CPU)
    assert n == sensor.n_sensors
    _assert_equal_inputs(dev, host)


def test_device_inputs_whole_domain_recording_equal_host_solver():
    from fullwave25_gb300.solver import Solver
    from fullwave25_gb300.workloads import plain_2d_problem

    grid, medium, source, sensor, _ = plain_2d_problem(shape=(40, 36), nt=60, seed=2)
    s = Solver("/tmp", grid, medium, source, sensor, pml_layer_thickness_px=6,
               n_transition_layer=6)
    host, hs = s.build_engine_inputs(record_whole_domain=True, sampling_modulus_time_whole_domain=4)
    dev, n = s.build_device_inputs(record_whole_domain=True, sampling_modulus_time_whole_domain=4,
                                   device=CPU)
    assert n == hs.n_sensors == int(np.prod(host.shape))
    _assert_equal_inputs(dev, host)


def test_device_inputs_reject_pml_without_transition_layer():
    from fullwave25_gb300.device_build import device_inputs

    g, med, src, sen, kw = _scenario("2d_small")
    kw["n_transition"] = 0
    with pytest.raises(ValueError, match="Transition layer"):
        device_inputs(g, med, src, sen, device=CPU, **kw)
