"""Host-side behaviour of the plugin mirror (no GPU): registry, the
reference's error behaviour, seeds, parameter traversal and state rotation."""
import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import scenes


def cpu_scene(two_state=True, albedo=0.8, D=4):
    dens = scenes.blob_density(D, 0)
    d = scenes.scene_dict(dens, albedo, res=8, two_state=two_state)
    return rcv.load_dict(d, device="cpu")


def test_plugin_names_registered():
    from recursive_control_variates_gb300.core import _KINDS

    for name in ("cv", "meta", "twostateprbvolpath", "twostateprb", "prbvolpath", "volpathsimple"):
        assert _KINDS[name] == "integrator"
    assert _KINDS["twostatemedium"] == "medium"


def test_volpathsimple_options():
    """Switches of plugins/volpathsimple.py:33-48 (all on by default) and its
    use as the `adjoint_integrator` of `cv` (experiments.py:131,245,364)."""
    v = rcv.load_dict({"type": "volpathsimple"})
    f = v.flags()
    assert (f.use_nee, f.use_drt, f.use_drt_subsampling, f.use_drt_mis) == (1, 1, 1, 1)
    v = rcv.load_dict({"type": "volpathsimple", "use_drt_mis": False, "use_nee": False, "max_depth": 12})
    f = v.flags()
    assert (f.use_nee, f.use_drt, f.use_drt_subsampling, f.use_drt_mis) == (0, 1, 1, 0)
    assert v.max_depth == 12 and "use_drt_mis = False" in v.to_string()
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath"},
                           "adjoint_integrator": {"type": "volpathsimple"}})
    assert type(integ.adjoint_integrator).__name__ == "VolpathSimpleIntegrator"
    assert v._checked_medium(cpu_scene(two_state=False)) is not None  # a plain medium is accepted


def test_cv_requires_two_state_integrator():
    with pytest.raises(ValueError, match="twostate"):
        rcv.load_dict({"type": "cv", "integrator": {"type": "prbvolpath"}})
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath", "max_depth": 16, "rr_depth": 16}})
    assert integ.warmup == 1 and integ.beta1 == 0.9 and integ.beta2 == 0.999
    assert integ.adjoint_integrator is integ.integrator
    assert integ.integrator.max_depth == 16


def test_meta_options():
    with pytest.raises(ValueError):
        rcv.load_dict({"type": "meta", "method": "cv_ps", "denoise": True, "integrator": {"type": "twostateprbvolpath"}})
    with pytest.raises(ValueError):
        rcv.load_dict({"type": "meta", "method": "bogus", "integrator": {"type": "twostateprbvolpath"}})
    m = rcv.load_dict({"type": "meta", "method": "cv_ps", "pre_update": True, "integrator": {"type": "twostateprbvolpath"}})
    assert m.pre_update and m.method == "cv_ps"


def test_check_scene_requires_two_state_medium():
    integ = rcv.load_dict({"type": "twostateprbvolpath"})
    with pytest.raises(RuntimeError, match="No TwoStateMedium"):
        integ.check_scene(cpu_scene(two_state=False))
    integ.check_scene(cpu_scene(two_state=True))


def test_unknown_plugin_and_unsupported_options():
    with pytest.raises(ValueError):
        rcv.load_dict({"type": "nope"})
    with pytest.raises(ValueError):
        rcv.load_dict({"type": "constant", "radiance": 2.0})
    dens = scenes.blob_density(4, 0)
    bad = scenes.medium_dict(dens, 0.8)
    bad["majorant_resolution_factor"] = -1
    with pytest.raises(ValueError):
        rcv.load_dict(bad, device="cpu")


def test_majorant_resolution_factor():
    """`majorant_resolution_factor` (experiments.py:70,187,306) is accepted on the
    heterogeneous media; the two-state medium reports and sets the factor of
    its states (plugins/twostatemedium.py:171-178)."""
    dens = scenes.blob_density(16, 0)
    m = scenes.medium_dict(dens, 0.8)
    m["majorant_resolution_factor"] = 8
    med = rcv.load_dict(m, device="cpu")
    assert med.majorant_resolution_factor() == 8 and med.c_struct().majorant_factor == 8
    scene = cpu_scene()
    tm = scene.named_shapes()["object"].interior_medium()
    assert tm.majorant_resolution_factor() == 0
    tm.set_majorant_resolution_factor(4)
    assert tm.majorant_resolution_factor() == 4 and tm.c_struct().majorant_factor == 4
    assert tm.old.majorant_factor == tm.incoming.majorant_factor == 4
    with pytest.raises(ValueError):
        tm.set_majorant_resolution_factor(-2)


def test_seed_rules():
    assert rcv.default_seed_grad(5) == rcv.sample_tea_32(5, 1)[0]
    scene = cpu_scene()
    integ = rcv.load_dict({"type": "twostateprbvolpath"})
    with pytest.raises(Exception, match="different"):
        rcv.render(scene, None, integ, seed=3, seed_grad=3, spp=4)


def test_traverse_keys_and_rotation():
    scene = cpu_scene(albedo=scenes.albedo_grid(4, 0))
    params = rcv.traverse(scene)
    assert set(params.keys()) == {scenes.DENSITY_KEY, scenes.ALBEDO_KEY}
    med = scene.named_shapes()["object"].interior_medium()
    first = med.new.density.clone()
    a = torch.full_like(first, 2.0)
    b = torch.full_like(first, 3.0)
    params[scenes.DENSITY_KEY] = a
    params.update()
    assert torch.equal(med.old.density, first) and torch.equal(med.new.density, a)
    params[scenes.DENSITY_KEY] = b
    params.update()
    assert torch.equal(med.old.density, a) and torch.equal(med.new.density, b)
    assert torch.equal(med.incoming.density, b)
    with pytest.raises(ValueError):
        params[scenes.DENSITY_KEY] = torch.zeros(2, 2, 2, 1)


def test_params_update_from_optimizer_keys():
    scene = cpu_scene()
    params = rcv.traverse(scene)

    class FakeOpt(dict):
        pass

    opt = FakeOpt({scenes.DENSITY_KEY: torch.full((4, 4, 4, 1), 1.0, requires_grad=True), "other": torch.zeros(1)})
    params.update(opt)
    assert params[scenes.DENSITY_KEY] is opt[scenes.DENSITY_KEY]
    assert scenes.DENSITY_KEY in params.differentiable()


def test_sensor_basis():
    scene = cpu_scene()
    s = scene.sensors()[0].c_struct()
    f = np.array(s.forward)
    r = np.array(s.right)
    u = np.array(s.up)
    assert np.allclose(f, [0, 0, -1], atol=1e-6)
    assert np.isclose(np.linalg.norm(r), np.tan(np.radians(22.5)), atol=1e-6)
    assert abs(float(f @ r)) < 1e-6 and abs(float(f @ u)) < 1e-6


def test_blob_generator_matches_specification():
    D = 16
    rho = scenes.blob_density(D, 0)[..., 0].astype(np.float64)
    rng = np.random.default_rng(0)
    c = rng.uniform(0.2, 0.8, (8, 3))
    s = rng.uniform(0.05, 0.15, 8)
    a = rng.uniform(5, 20, 8)
    i, j, k = 3, 7, 11  # z, y, x
    x = np.array([k + 0.5, j + 0.5, i + 0.5]) / D
    expect = sum(a[n] * np.exp(-np.sum((x - c[n]) ** 2) / (2 * s[n] ** 2)) for n in range(8))
    assert np.isclose(rho[i, j, k], expect, rtol=1e-6)
