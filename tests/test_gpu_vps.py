"""GPU parity of the volpathsimple integrator (plugins/volpathsimple.py of
the reference) through the C ABI, against the oracle's restatement on the
same seeded inputs.

Tolerances as for the two-state tracer: the kernels follow the oracle's
per-path float32 operation sequence, so primal pixels are compared for exact
equality on >= 99.9 % of pixels (and means to 1e-5 relative); gradients
accumulate with float atomics in a different order than the oracle's double
sums, compared at 2e-5 relative L2 (density and albedo)."""
import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import scenes

from test_gpu_volume import frac_equal, make_scene, oracle_scene

pytestmark = pytest.mark.gpu

FLAG_CASES = [{}, {"use_drt": False}, {"use_drt_subsampling": False}, {"use_drt_mis": False}, {"use_nee": False}]


def vps_integrator(flags, max_depth=8):
    d = {"type": "volpathsimple", "max_depth": max_depth, "rr_depth": max_depth}
    d.update(flags)
    return rcv.load_dict(d)


def with_factor(med, factor):
    med.set_majorant_resolution_factor(factor)
    return med


@pytest.mark.parametrize("factor", [0, 4])
@pytest.mark.parametrize("flags", [{}, {"use_nee": False}])
@pytest.mark.parametrize("albedo_grid", [False, True])
def test_vps_primal_matches_oracle(cuda, oracle, flags, factor, albedo_grid):
    scene, med, grids = make_scene(cuda, albedo_grid=albedo_grid)
    with_factor(med, factor)
    img = vps_integrator(flags).render(scene, 0, seed=9, spp=4).cpu().numpy()
    ref = oracle.vps_render(oracle_scene(oracle, scene, grids, 8, albedo_grid, factor), seed=9, spp=4, flags=flags)
    assert frac_equal(img, ref) >= 0.999
    np.testing.assert_allclose(img.mean(), ref.mean(), rtol=1e-5)


@pytest.mark.parametrize("flags", FLAG_CASES)
def test_vps_adjoint_matches_oracle(cuda, oracle, flags):
    scene, med, grids = make_scene(cuda, res=32)
    params = rcv.traverse(scene)
    rng = np.random.default_rng(5)
    gimg = rng.normal(0, 1, (32, 32, 3)).astype(np.float32)
    grads = vps_integrator(flags).render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=31, spp=4)
    gd = grads[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    od, _ = oracle.vps_backward(oracle_scene(oracle, scene, grids, 8, False), seed=31, spp=4, grad_img=gimg,
                                flags=flags)
    assert np.linalg.norm(od) > 0
    assert np.linalg.norm(gd - od) <= 2e-5 * np.linalg.norm(od)


@pytest.mark.parametrize("factor", [0, 4])
def test_vps_adjoint_albedo_grid_and_supergrid(cuda, oracle, factor):
    scene, med, grids = make_scene(cuda, res=32, albedo_grid=True)
    with_factor(med, factor)
    params = rcv.traverse(scene)
    rng = np.random.default_rng(6)
    gimg = rng.normal(0, 1, (32, 32, 3)).astype(np.float32)
    grads = vps_integrator({}).render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=8, spp=4)
    gd = grads[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    ga = grads[scenes.ALBEDO_KEY].cpu().numpy().astype(np.float64)
    od, oa = oracle.vps_backward(oracle_scene(oracle, scene, grids, 8, True, factor), seed=8, spp=4, grad_img=gimg)
    assert np.linalg.norm(gd - od) <= 2e-5 * np.linalg.norm(od)
    assert np.linalg.norm(ga - oa) <= 2e-5 * np.linalg.norm(oa)


@pytest.mark.parametrize("flags", [{}, {"use_drt": False}])
@pytest.mark.parametrize("max_depth,rr_depth", [(16, 2), (-1, 3), (0, 0)])
def test_vps_roulette_and_depth_limits_match_oracle(cuda, oracle, flags, max_depth, rr_depth):
    """Russian roulette below max_depth (plugins/volpathsimple.py:131),
    unlimited depth ended by the roulette, and max_depth 0: primal and
    adjoint against the oracle."""
    from test_gpu_volume import _oracle_scene_opts

    scene, med, grids = make_scene(cuda, res=32, albedo_grid=True)
    params = rcv.traverse(scene)
    d = {"type": "volpathsimple", "max_depth": max_depth, "rr_depth": rr_depth}
    d.update(flags)
    integ = rcv.load_dict(d)
    osc = _oracle_scene_opts(oracle, scene, grids, max_depth, rr_depth, False)
    img = integ.render(scene, 0, seed=13, spp=4).cpu().numpy()
    ref = oracle.vps_render(osc, seed=13, spp=4, flags=flags)
    assert frac_equal(img, ref) >= 0.999
    np.testing.assert_allclose(img.mean(), ref.mean(), rtol=1e-5)
    rng = np.random.default_rng(7)
    gimg = rng.normal(0, 1, (32, 32, 3)).astype(np.float32)
    grads = integ.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=14, spp=4)
    od, oa = oracle.vps_backward(osc, seed=14, spp=4, grad_img=gimg, flags=flags)
    gd = grads[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    ga = grads[scenes.ALBEDO_KEY].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(od) > 0
    assert np.linalg.norm(gd - od) <= 2e-5 * np.linalg.norm(od)
    if np.linalg.norm(oa) > 0:
        assert np.linalg.norm(ga - oa) <= 2e-5 * np.linalg.norm(oa)
    else:
        assert float(np.abs(ga).max()) == 0.0


def test_cv_with_volpathsimple_adjoint(cuda):
    """The grid experiments' pairing (experiments.py:131,245,364): a `cv`
    integrator over the two-state tracer whose gradients come from
    volpathsimple; the adjoint call is delegated unchanged."""
    scene, med, grids = make_scene(cuda, res=24)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8},
                           "adjoint_integrator": {"type": "volpathsimple", "max_depth": 8, "rr_depth": 8}})
    g = torch.ones((24, 24, 3), device=cuda)
    a = integ.render_backward(scene, params, g, 0, seed=4, spp=2)[scenes.DENSITY_KEY]
    b = integ.adjoint_integrator.render_backward(scene, params, g, 0, seed=4, spp=2)[scenes.DENSITY_KEY]
    assert torch.isfinite(a).all() and float(a.abs().sum()) > 0
    # float atomics: the two calls add in different orders
    assert float((a - b).norm()) <= 1e-5 * float(b.norm())
