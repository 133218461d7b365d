"""Surface form (twostateprb + twostate BSDF): oracle invariants and adjoint
consistency on the CPU; GPU parity of the surface kernels with the oracle.

Tolerances: the primal tracers follow the oracle's float operations, so
>= 99.9 % of pixels must be bit-identical; the texture gradient accumulates
with float atomics: 2e-5 relative L2 against the oracle (double)."""
import ctypes as C

import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import scenes


def oracle_surface(O, tex_old, tex_new, res, seed=0, max_depth=6, rr_depth=3):
    cam = O.camera_basis(res, res, *scenes.SURFACE_CAMERA)
    return O.SurfaceScene(cam, tex_old, tex_new, scenes.surface_spheres(seed), (0.0, 3.0, 0.0), (0.5, 0.5),
                          (15.0, 15.0, 15.0), plane_half=2.0, max_depth=max_depth, rr_depth=rr_depth)


# ------------------------------------------------------------------- CPU
def test_surface_equal_states(oracle):
    tex = scenes.value_noise(32, 2)
    sc = oracle_surface(oracle, tex, tex, 24)
    H, F = oracle.surface_render_twostates(sc, seed=3, spp=8)
    S = oracle.surface_render(sc, seed=3, spp=8)
    assert np.array_equal(F, S)
    # old == new: the old throughput is eval_old / pdf, the new one the
    # sampled weight; they agree to float rounding (plugins/twostatepath.py:328-333)
    np.testing.assert_allclose(H, F, rtol=2e-6, atol=1e-7)
    assert F.mean() > 0.02


def test_surface_adjoint_matches_two_state_differences(oracle):
    res, T = 24, 8
    base = scenes.value_noise(T, 5)
    rng = np.random.default_rng(1)
    dl = rng.normal(0, 1, (res, res, 3)).astype(np.float32)
    sc = oracle_surface(oracle, base, base, res)
    runs = np.array([oracle.surface_backward(sc, seed=50 + s, spp=64, grad_img=dl) for s in range(8)])
    delta = np.zeros_like(base)
    delta[2:6, 2:6, :] = 1.0  # a patch in the middle of the plane
    h = 0.05
    s2 = oracle_surface(oracle, base - h * delta, base + h * delta, res)
    est = []
    for seed in range(8):
        H, F = oracle.surface_render_twostates(s2, seed=9 + seed, spp=64)
        est.append(float(((F.astype(np.float64) - H) * dl).sum() / (2 * h)))
    fd, fd_se = np.mean(est), np.std(est) / np.sqrt(len(est))
    proj = (runs * delta).sum(axis=(1, 2, 3))
    adj, adj_se = proj.mean(), proj.std() / np.sqrt(len(proj))
    assert abs(fd - adj) < 4 * np.hypot(fd_se, adj_se) + 1e-4, (fd, fd_se, adj, adj_se)
    assert abs(adj) > 3 * adj_se  # the check is not vacuous


def test_surface_host_errors():
    tex = np.full((8, 8, 3), 0.5, np.float32)
    sc = rcv.load_dict(scenes.surface_scene_dict(tex, res=16), device="cpu")
    integ = rcv.load_dict({"type": "twostateprb", "max_depth": 8})
    integ.check_scene(sc)
    d = scenes.surface_scene_dict(tex, res=16)
    d["plane"]["bsdf"] = {"type": "diffuse", "reflectance": 0.5}
    with pytest.raises(ValueError):
        rcv.load_dict(d, device="cpu")
    cube = rcv.load_dict(scenes.scene_dict(scenes.blob_density(4, 0), 0.8, res=8), device="cpu")
    with pytest.raises(ValueError, match="TwoStateMedium"):
        rcv.load_dict({"type": "twostateprb"}).check_scene(cube)
    assert rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprb"}}).integrator.max_depth == 6


# ------------------------------------------------------------------- GPU
def gpu_scene(device, tex_old, tex_new, res, seed=0):
    scene = rcv.load_dict(scenes.surface_scene_dict(tex_new, res=res, seed=seed), device=device)
    b = scene.named_shapes()["plane"].bsdf
    b.old.texture.data.copy_(torch.from_numpy(np.ascontiguousarray(tex_old)))
    b._dirty = True
    return scene


@pytest.mark.gpu
@pytest.mark.parametrize("batch", [1, 64])
def test_surface_two_state_matches_oracle(cuda, oracle, batch):
    res = 40
    told, tnew = scenes.value_noise(32, 1), scenes.value_noise(32, 2)
    scene = gpu_scene(cuda, told, tnew, res)
    integ = rcv.load_dict({"type": "twostateprb", "max_depth": 6, "rr_depth": 3, "batch": batch})
    H, F = integ.render_twostates(scene, 0, seed=4, spp=8)
    S = integ.render(scene, 0, seed=4, spp=8)
    Ho, Fo = oracle.surface_render_twostates(oracle_surface(oracle, told, tnew, res), seed=4, spp=8)
    H, F, S = H.cpu().numpy(), F.cpu().numpy(), S.cpu().numpy()
    for a, b in ((H, Ho), (F, Fo), (S, Fo)):
        assert np.mean(np.all(a == b, axis=-1)) >= 0.999
    assert not np.array_equal(H, F)


@pytest.mark.gpu
@pytest.mark.parametrize("adjoint,per_path", [("tape", 0), ("tape", 1), ("tape", 4), ("replay", 0)])
def test_surface_adjoint_matches_oracle(cuda, oracle, adjoint, per_path):
    """The texture gradient from the tape of texture vertices (16 slots per
    path; 1 and 4: most paths lose vertices and are replayed) and from the
    second tracing pass, against the oracle and against each other (the
    same vertex terms; only the order of float additions differs)."""
    res = 32
    tex = scenes.value_noise(16, 3)
    scene = gpu_scene(cuda, tex, tex, res)
    params = rcv.traverse(scene)
    gimg = np.random.default_rng(2).normal(0, 1, (res, res, 3)).astype(np.float32)
    grads = {}
    for mode, pp in ((adjoint, per_path), ("replay", 0)):
        integ = rcv.load_dict({"type": "twostateprb", "max_depth": 6, "rr_depth": 3, "adjoint": mode,
                               "tape_events_per_path": pp})
        g = integ.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=21, spp=16)
        grads[mode] = g[scenes.TEXTURE_KEY].cpu().numpy().astype(np.float64)
    g = grads[adjoint]
    go = oracle.surface_backward(oracle_surface(oracle, tex, tex, res), seed=21, spp=16, grad_img=gimg)
    assert np.linalg.norm(g - go) <= 2e-5 * np.linalg.norm(go)
    assert np.linalg.norm(g - grads["replay"]) <= 1e-6 * np.linalg.norm(grads["replay"])


@pytest.mark.gpu
def test_surface_cv_optimisation(cuda):
    res, T = 64, 32
    target_tex = scenes.value_noise(T, 7)
    ref_scene = gpu_scene(cuda, target_tex, target_tex, res)
    base = rcv.load_dict({"type": "twostateprb", "max_depth": 8, "rr_depth": 5})
    target = base.render(ref_scene, 0, seed=17843, spp=256)
    init = np.full_like(target_tex, 0.5)
    scene = gpu_scene(cuda, init, init, res)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprb", "max_depth": 8, "rr_depth": 5}})
    opt = rcv.ad.Adam(lr=0.05)
    opt[scenes.TEXTURE_KEY] = init
    opt.set_bounds(scenes.TEXTURE_KEY, 0.0, 1.0)
    params.update(opt)
    params.update(opt)
    err0 = float(np.abs(init - target_tex).mean())
    for it in range(60):
        params.update(opt)
        img = rcv.render(scene, params, integrator=integ, seed=it, spp=8)
        rcv.l2_loss(img, target).backward()
        opt.step()
    err = float(np.abs(opt[scenes.TEXTURE_KEY].detach().cpu().numpy() - target_tex).mean())
    assert err < 0.8 * err0, (err, err0)


def test_surface_forward_is_the_adjoint_transposed(oracle):
    """Surface forward mode (oracle): <w, J t> = <J^T w, t> for the same seed."""
    res, T = 24, 16
    tex = np.random.default_rng(4).uniform(0.2, 0.9, (T, T, 3)).astype(np.float32)
    sc = oracle_surface(oracle, tex, tex, res)
    rng = np.random.default_rng(5)
    w = rng.normal(0, 1, (res, res, 3)).astype(np.float32)
    t = rng.normal(0, 1, (T, T, 3)).astype(np.float32)
    fw = oracle.surface_forward(sc, seed=9, spp=8, tangent=t).astype(np.float64)
    g = oracle.surface_backward(sc, seed=9, spp=8, grad_img=w)
    lhs, rhs = float((w * fw).sum()), float((g * t).sum())
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs)), (lhs, rhs)


@pytest.mark.gpu
def test_surface_forward_matches_oracle(cuda, oracle):
    res, T = 32, 16
    tex = np.random.default_rng(6).uniform(0.2, 0.9, (T, T, 3)).astype(np.float32)
    scene = gpu_scene(cuda, tex, tex, res)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "twostateprb", "max_depth": 6, "rr_depth": 3})
    t = np.random.default_rng(7).normal(0, 1, (T, T, 3)).astype(np.float32)
    fw = integ.render_forward(scene, params, 0, seed=11, spp=8,
                              tangents={scenes.TEXTURE_KEY: torch.from_numpy(t).to(cuda)})
    ofw = oracle.surface_forward(oracle_surface(oracle, tex, tex, res), seed=11, spp=8, tangent=t).astype(np.float64)
    f = fw.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(ofw) > 0
    assert np.linalg.norm(f - ofw) <= 2e-5 * np.linalg.norm(ofw)
