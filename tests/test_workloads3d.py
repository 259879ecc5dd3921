"""The torch (device-side) 3D workload builder uses the same PML arithmetic as the host builder
that is byte-checked against the reference."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_torch_ramp_equals_numpy_ramp():
    from fullwave25_gb300.pml import ramp_axis
    from fullwave25_gb300.workloads3d import ramp_axis_t

    rng = np.random.default_rng(1)
    base = rng.uniform(1e4, 6e4, size=(40, 38, 36))
    for kind, thick, off in (("polynomial", 12, 0), ("linear", 12, 0), ("cosine", 6, 6)):
        a = base.copy()
        t = torch.as_tensor(base.copy())
        for axis in range(3):
            a = ramp_axis(a, 123.0, axis, thickness=thick, offset=off, kind=kind)
            t = ramp_axis_t(t, 123.0, axis, thickness=thick, offset=off, kind=kind)
        np.testing.assert_allclose(t.numpy(), a, rtol=1e-15, atol=0)


def test_torch_pml_maps_equal_host_builder():
    from fullwave25_gb300.grid import Grid
    from fullwave25_gb300.medium import MediumRelaxationMaps
    from fullwave25_gb300.pml import PMLBuilder, extend_map
    from fullwave25_gb300.source import Sensor, Source
    from fullwave25_gb300.workloads3d import extend_edge, pml_relaxation_maps_t
    from golden_io import load_case

    z = load_case("3d_small")
    shape = tuple(int(v) for v in z["shape"])
    g = Grid.from_cells(shape, f0=float(z["f0"]), nt=int(z["nt"]), ppw=int(z["ppw"]),
                        cfl=float(z["cfl"]))
    relax = {k[6:]: z[k] for k in z.files if k.startswith("relax/")}
    med = MediumRelaxationMaps(g, z["c"], z["rho"], z["beta"], relax)
    b = PMLBuilder(g, med, Source(z["p0"], z["src_mask"]), Sensor(z["sens_mask"]),
                   n_pml_layer=int(z["n_pml"]), n_transition_layer=int(z["n_transition"]))
    ref = b.run().relaxation_param_dict_for_fw2
    nb = b.num_boundary_points
    params = {k: extend_edge(torch.as_tensor(v), nb) for k, v in med.relaxation_param_dict.items()}
    np.testing.assert_array_equal(params["d_x1_nu1"].numpy(),
                                  extend_map(med.relaxation_param_dict["d_x1_nu1"], nb))
    got = pml_relaxation_maps_t(params, n_pml=int(z["n_pml"]), n_transition=int(z["n_transition"]),
                                dt=b.extended_grid.dt, c0=b.extended_grid.c0, dx=b.extended_grid.dx)
    for k in ("kappa_u", "kappa_x", "a_pml_u1", "b_pml_u1", "a_pml_x2", "b_pml_x2"):
        np.testing.assert_allclose(got[k].numpy(), ref[k], rtol=1e-13, atol=1e-300)


def test_small_plain_3d_workload_on_cpu():
    from fullwave25_gb300.workloads3d import plain_3d_host_sample

    inp = plain_3d_host_sample(edge=24, nt=50)
    inp.validate()
    assert inp.shape == (24 + 48,) * 3
    assert inp.icc.shape[0] == 24 * 8 and inp.outc.shape[0] == 16 * 16
    assert np.isfinite(np.stack([v for v in inp.maps.values()])).all()
    assert inp.dcmap.min() == 0 and inp.dcmap.max() == inp.dmap.shape[2] - 1


def test_anisotropic_host_builder_gives_every_direction_the_same_maps():
    """The anisotropic PML builder ramps every direction's maps along every axis from the same
    gradient / divergence parameters, so the per-direction sets equal the first direction's:
    what the device-side anisotropic workload replicates."""
    from fullwave25_gb300.grid import Grid
    from fullwave25_gb300.medium import MediumRelaxationMaps
    from fullwave25_gb300.pml import PMLBuilder
    from fullwave25_gb300.source import Sensor, Source
    from golden_io import load_case

    z = load_case("3d_small")
    shape = tuple(int(v) for v in z["shape"])
    g = Grid.from_cells(shape, f0=float(z["f0"]), nt=int(z["nt"]), ppw=int(z["ppw"]),
                        cfl=float(z["cfl"]))
    relax = {k[6:]: z[k] for k in z.files if k.startswith("relax/")}
    med = MediumRelaxationMaps(g, z["c"], z["rho"], z["beta"], relax)
    med.use_isotropic_relaxation = False
    b = PMLBuilder(g, med, Source(z["p0"], z["src_mask"]), Sensor(z["sens_mask"]),
                   n_pml_layer=int(z["n_pml"]), n_transition_layer=int(z["n_transition"]),
                   use_isotropic_relaxation=False)
    out = b.run().relaxation_param_dict_for_fw2
    for first, others in (("u", ("w", "v")), ("x", ("y", "z"))):
        for o in others:
            for key in ("kappa_{}", "a_pml_{}1", "b_pml_{}1", "a_pml_{}2", "b_pml_{}2"):
                np.testing.assert_array_equal(out[key.format(o)], out[key.format(first)])


def test_physics_variants_of_the_3d_workload():
    from fullwave25_gb300.exponential import body_mask, db_mhz_cm_to_a_exp
    from fullwave25_gb300.grid import Grid
    from fullwave25_gb300.inputs import anisotropic_extra_maps
    from fullwave25_gb300.workloads3d import exp_attenuation_t, plain_3d_host_sample

    iso = plain_3d_host_sample(edge=24, nt=50)
    an = plain_3d_host_sample(edge=24, nt=50, physics="aniso")
    an.validate()
    assert set(an.maps) == set(iso.maps) | set(anisotropic_extra_maps(3))
    np.testing.assert_array_equal(an.maps["kappav"], iso.maps["kappau"])
    np.testing.assert_array_equal(an.maps["bpmlz2"], iso.maps["bpmlx2"])
    ex = plain_3d_host_sample(edge=24, nt=50, physics="exp")
    ex.validate()
    assert set(ex.maps) == {"c", "rho", "K", "beta", "a_exp"}
    a = ex.maps["a_exp"]
    assert a.shape == ex.shape and 0 <= a.min() and a.max() < 1 and a[36, 36, 36] > 0.99
    # the device formula against the host builder's
    g = Grid.from_cells((20, 18, 16), f0=2e6, nt=10, ppw=10, cfl=0.2)
    alpha = np.random.default_rng(0).uniform(0.2, 1.2, size=(20, 18, 16))
    ref = db_mhz_cm_to_a_exp(alpha, g) * (1 - body_mask(alpha.shape, 5))
    got = exp_attenuation_t(torch.as_tensor(alpha), g, 5).numpy()
    np.testing.assert_allclose(got, ref, rtol=1e-14, atol=1e-300)
