"""The two-state render and the adjoint's radiance pass in one persistent
launch (rcv_render_twostates_volume_and_adjoint_radiance, csrc/rcv_pair.cu).

Each tracer keeps its own queue, pixel order, random streams and outputs, so
the images must be bit-identical to those of the two-state call alone, and
the gradient that the replay call completes from the paired radiance pass
must equal the one-call adjoint (float atomics in another order: 1e-6
relative L2) and the oracle (2e-5).  Event counting and the replay adjoint
take the two launches one after the other inside the same call."""
import ctypes as C

import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import _lib, scenes

from test_envmap import gpu_env_scene, oracle_env_scene, random_map
from test_gpu_volume import make_scene, oracle_scene

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def host(g):
    return {k: v.detach().cpu().numpy().astype(np.float64) for k, v in g.items()}


CASES = {
    "plain": {},
    "supergrid": {"factor": 4},
    "envmap": {"env": True},
    "lost_paths": {"props": {"tape_events_per_path": 2}},
    "counting": {"props": {"count_events": True}},
    "replay_adjoint": {"props": {"adjoint": "replay"}},
}


@pytest.mark.parametrize("case", list(CASES))
def test_paired_launch_matches_separate_calls(cuda, oracle, case):
    c = CASES[case]
    res = 32
    if c.get("env"):
        env, scale = random_map(), 1.3
        scene, grids = gpu_env_scene(cuda, env, scale, res=res)
        osc = oracle_env_scene(oracle, scene, grids, env, scale)
    else:
        scene, med, grids = make_scene(cuda, albedo_grid=True, D=24 if c.get("factor") else 16, res=res)
        if c.get("factor"):
            med.set_majorant_resolution_factor(c["factor"])
        osc = oracle_scene(oracle, scene, grids, 8, True, c.get("factor", 0))
    props = {"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8, **c.get("props", {})}
    integ = rcv.load_dict(props)
    params = rcv.traverse(scene)
    gimg = np.random.default_rng(3).normal(0, 1, (res, res, 3)).astype(np.float32)
    g = torch.from_numpy(gimg).to(cuda)

    H0, F0 = integ.render_twostates(scene, 0, seed=9, spp=4)
    assert integ.last_primal_call == "rcv_render_twostates_volume"
    full = host(integ.render_backward(scene, params, g, 0, seed=5, spp=6))
    assert integ.last_adjoint_call == "rcv_render_backward_volume"

    launch = integ.prefetch_adjoint(scene, 0, seed=5, spp=6)
    H, F = integ.render_twostates(scene, 0, seed=9, spp=4)
    assert integ.last_primal_call == "rcv_render_twostates_volume_and_adjoint_radiance"
    launch()  # already ran in the paired launch: nothing to do
    paired = host(integ.render_backward(scene, params, g, 0, seed=5, spp=6))
    assert integ.last_adjoint_call == "rcv_render_backward_replay"
    assert torch.equal(H, H0) and torch.equal(F, F0)

    od, oa = oracle.backward(osc, seed=5, spp=6, grad_img=gimg)
    gd = paired[scenes.DENSITY_KEY][..., 0]
    assert np.linalg.norm(od) > 0
    assert rel_l2(gd, full[scenes.DENSITY_KEY][..., 0]) <= 1e-6
    assert rel_l2(gd, od) <= 2e-5, rel_l2(gd, od)
    assert rel_l2(paired[scenes.ALBEDO_KEY], full[scenes.ALBEDO_KEY]) <= 1e-6
    assert rel_l2(paired[scenes.ALBEDO_KEY], oa) <= 2e-5


def test_pairing_off_and_mismatched_requests(cuda):
    """pair_adjoint False keeps the side-stream launch; a radiance pass
    prepared for another sensor or medium state is not paired."""
    scene, med, grids = make_scene(cuda, albedo_grid=True, res=24)
    params = rcv.traverse(scene)
    g = torch.randn((24, 24, 3), device=cuda)
    off = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8, "pair_adjoint": False})
    launch = off.prefetch_adjoint(scene, 0, seed=5, spp=4)
    H0, F0 = off.render_twostates(scene, 0, seed=9, spp=4)
    assert off.last_primal_call == "rcv_render_twostates_volume"
    launch()
    a = host(off.render_backward(scene, params, g, 0, seed=5, spp=4))
    assert off.last_adjoint_call == "rcv_render_backward_replay"

    on = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    launch = on.prefetch_adjoint(scene, 0, seed=5, spp=4)
    launch()  # launched before the render: the render runs alone
    H, F = on.render_twostates(scene, 0, seed=9, spp=4)
    assert on.last_primal_call == "rcv_render_twostates_volume"
    assert torch.equal(H, H0) and torch.equal(F, F0)
    b = host(on.render_backward(scene, params, g, 0, seed=5, spp=4))
    assert on.last_adjoint_call == "rcv_render_backward_replay"
    assert rel_l2(b[scenes.DENSITY_KEY], a[scenes.DENSITY_KEY]) <= 1e-6

    # the medium changes between the request and the render: not paired,
    # and the backward pass runs in full on the new state
    launch = on.prefetch_adjoint(scene, 0, seed=5, spp=4)
    med.new.density.mul_(1.01)
    med._dirty = True
    on.render_twostates(scene, 0, seed=9, spp=4)
    assert on.last_primal_call == "rcv_render_twostates_volume"
    launch()
    on.render_backward(scene, params, g, 0, seed=5, spp=4)
    assert on.last_adjoint_call == "rcv_render_backward_volume"

    # separate_tracers is 0 or 1
    sensor = scene.sensors()[0]
    o = on.options(scene)
    o.separate_tracers = 2
    m = med.prepare(torch.cuda.current_stream(cuda).cuda_stream)
    H = torch.empty((24, 24, 3), device=cuda)
    F = torch.empty_like(H)
    rc = _lib.load().rcv_render_twostates_volume_and_adjoint_radiance(
        C.byref(m), C.byref(sensor.c_struct()), C.byref(o), 9, 4, H.data_ptr(), F.data_ptr(),
        on.scratch(cuda, sensor, 4, _lib.MODE_TWOSTATE), 5, 4, on.adjoint_scratch(cuda, sensor, 4), None,
        torch.cuda.current_stream(cuda).cuda_stream)
    assert rc == _lib.RCV_ERR_INVALID
    assert b"separate_tracers" in _lib.load().rcv_last_error()


def test_paired_step_through_the_public_api(cuda):
    """rcv.render with the cv integrator: the forward pass pairs the
    radiance pass with the two-state render; the gradient equals that of
    the same step with the pairing off."""
    grads = []
    for pair in (True, False):
        scene, med, grids = make_scene(cuda, albedo_grid=True, res=24)
        params = rcv.traverse(scene)
        opt = rcv.ad.Adam(lr=0.01)
        opt[scenes.DENSITY_KEY] = params[scenes.DENSITY_KEY]
        params.update(opt)
        inner = {"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8, "pair_adjoint": pair}
        integ = rcv.load_dict({"type": "cv", "integrator": inner})
        img = rcv.render(scene, params, integrator=integ, seed=4, spp=4, spp_grad=8)
        (img * torch.linspace(-1, 1, img.numel(), device=cuda).reshape(img.shape)).sum().backward()
        expect = "rcv_render_twostates_volume_and_adjoint_radiance" if pair else "rcv_render_twostates_volume"
        assert integ.integrator.last_primal_call == expect
        assert integ.integrator.last_adjoint_call == "rcv_render_backward_replay"
        grads.append(opt[scenes.DENSITY_KEY].grad.double().cpu().numpy())
    assert np.linalg.norm(grads[0]) > 0
    assert rel_l2(grads[0], grads[1]) <= 1e-6
