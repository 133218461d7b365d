"""Environment map emitter (the reference's `envmap`, experiments.py:81-85,
195-199, 315-319): the oracle's map primitives checked against their
definitions on the CPU (arctangent, pdf normalisation, unbiased importance
sampling, agreement with the constant environment), and the CUDA tracers
against the oracle on the GPU (images bit-identical on >= 99.9 % of pixels,
gradients and forward derivatives within 2e-5 relative L2, as for the
constant environment)."""
import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import scenes


def random_map(h=12, w=24, seed=0):
    """A smooth map with a bright sun-like spot (strongly non-uniform)."""
    rng = np.random.default_rng(seed)
    img = rng.uniform(0.2, 1.0, (h, w, 3)).astype(np.float32)
    img[h // 4, w // 3] = [30.0, 28.0, 20.0]
    img[h - 2, 2] = [0.0, 0.0, 0.0]
    return img


def uniform_dirs(n, seed=1):
    rng = np.random.default_rng(seed)
    z = rng.uniform(-1, 1, n)
    phi = rng.uniform(0, 2 * np.pi, n)
    r = np.sqrt(1 - z * z)
    return np.stack([r * np.cos(phi), z, r * np.sin(phi)], axis=1).astype(np.float32)


def env_scene(O, env, scale=1.0, res=8, dens=None):
    cam = O.camera_basis(res, res)
    d = scenes.blob_density(8, 3)[..., 0] if dens is None else dens
    return O.Scene(cam, d, d, albedo_const=0.8, max_depth=8, envmap=env, envmap_scale=scale)


# ------------------------------------------------------------------- CPU
def test_arctangent_and_uv(oracle):
    rng = np.random.default_rng(3)
    for y, x in rng.normal(0, 1, (2000, 2)).astype(np.float32):
        assert abs(oracle.atan2(y, x) - np.arctan2(np.float64(y), np.float64(x))) < 4e-7
    for y, x in ((0.0, 1.0), (1.0, 0.0), (0.0, -1.0), (-1.0, 0.0), (1e-30, -1.0)):
        assert abs(oracle.atan2(y, x) - np.arctan2(y, x)) < 4e-7
    d = uniform_dirs(5000)
    uvs = oracle.env_uv(d)
    u_ref = np.mod(np.arctan2(d[:, 0].astype(np.float64), -d[:, 2]) / (2 * np.pi), 1.0)
    v_ref = np.arccos(np.clip(d[:, 1].astype(np.float64), -1, 1)) / np.pi
    du = np.abs(uvs[:, 0] - u_ref)
    assert np.all(np.minimum(du, 1 - du) < 2e-6) and np.all(np.abs(uvs[:, 1] - v_ref) < 2e-6)
    assert np.all((uvs[:, 0] >= 0) & (uvs[:, 0] < 1))


def test_pdf_is_normalised_and_matches_samples(oracle):
    env = random_map()
    sc = env_scene(oracle, env)
    # integral of the pdf over the sphere on a fine (u, v) midpoint grid:
    # pdf * sin(theta) is piecewise constant in (u, v), so the sum is exact
    # up to the cells the grid lines cut
    nu, nv = 960, 480
    u, v = np.meshgrid((np.arange(nu) + 0.5) / nu, (np.arange(nv) + 0.5) / nv)
    th, ph = np.pi * v.ravel(), 2 * np.pi * u.ravel()
    d = np.stack([np.sin(th) * np.sin(ph), np.cos(th), -np.sin(th) * np.cos(ph)], axis=1).astype(np.float32)
    _, pdf = oracle.env_eval(sc, d)
    integral = float(np.sum(pdf.astype(np.float64) * np.sin(th)) * (np.pi / nv) * (2 * np.pi / nu))
    assert abs(integral - 1.0) < 1e-4, integral
    u = np.random.default_rng(5).uniform(0, 1, (20000, 2)).astype(np.float32)
    dirs, le, ps = oracle.env_sample(sc, u)
    np.testing.assert_allclose(np.linalg.norm(dirs, axis=1), 1.0, atol=2e-6)
    le2, pdf2 = oracle.env_eval(sc, dirs)
    # the pdf looked up at the sampled direction is the sampled texel's
    # (except on texel edges), the radiance the same bilinear value
    assert np.mean(np.isclose(ps, pdf2, rtol=1e-4)) > 0.99
    assert np.mean(np.all(np.isclose(le, le2, rtol=1e-4, atol=1e-6), axis=1)) > 0.99
    assert float(ps.min()) > 0.0  # the black texel is never sampled


def test_importance_sampling_is_unbiased(oracle):
    """E[Le / pdf] over sampled directions = the integral of Le over the
    sphere, estimated independently with uniform directions."""
    env = random_map()
    sc = env_scene(oracle, env, scale=1.5)
    u = np.random.default_rng(7).uniform(0, 1, (400000, 2)).astype(np.float32)
    _, le, ps = oracle.env_sample(sc, u)
    est = le.astype(np.float64) / ps[:, None]
    d = uniform_dirs(400000, seed=8)
    le_u, _ = oracle.env_eval(sc, d)
    ref = le_u.astype(np.float64) * 4 * np.pi
    for c in range(3):
        se = np.hypot(est[:, c].std() / np.sqrt(len(est)), ref[:, c].std() / np.sqrt(len(ref)))
        assert abs(est[:, c].mean() - ref[:, c].mean()) < 4 * se, (c, est[:, c].mean(), ref[:, c].mean(), se)
    # importance sampling has the lower variance on a peaked map
    assert est[:, 0].std() < ref[:, 0].std()


def test_constant_map_matches_constant_environment(oracle):
    """A map of radiance 1 everywhere lights the medium like the constant
    environment (other samples, same expectation)."""
    res, spp = 12, 1024
    cam = oracle.camera_basis(res, res)
    d = scenes.blob_density(8, 3)[..., 0] * 0.5
    const = oracle.Scene(cam, d, d, albedo_const=0.8, max_depth=8)
    mapped = oracle.Scene(cam, d, d, albedo_const=0.8, max_depth=8, envmap=np.ones((6, 12, 3), np.float32))
    a = np.stack([oracle.render(const, seed=s, spp=spp) for s in range(4)]).astype(np.float64)
    b = np.stack([oracle.render(mapped, seed=100 + s, spp=spp) for s in range(4)]).astype(np.float64)
    ma, mb = a.mean(axis=(1, 2, 3)), b.mean(axis=(1, 2, 3))
    se = np.hypot(ma.std(ddof=1), mb.std(ddof=1)) / 2
    assert abs(ma.mean() - mb.mean()) < max(4 * se, 2e-3), (ma.mean(), mb.mean(), se)
    # pixels that see the environment directly are exactly 1
    corner_a, corner_b = a[:, 0, 0], b[:, 0, 0]
    assert np.all(corner_a == 1.0) and np.all(np.abs(corner_b - 1.0) < 1e-6)


def test_envmap_adjoint_matches_finite_differences(oracle):
    """Under a peaked map the oracle's path-replay adjoint still matches
    central differences of the two-state tracer."""
    res, D = 12, 8
    cam = oracle.camera_basis(res, res)
    env = random_map()
    theta = scenes.blob_density(D, 4)[..., 0] * 0.5
    w = np.random.default_rng(0).normal(0, 1, (res, res, 3)).astype(np.float32)
    sc = oracle.Scene(cam, theta, theta, albedo_const=0.8, max_depth=6, envmap=env)
    runs = np.array([oracle.backward(sc, seed=100 + s, spp=64, grad_img=w)[0] for s in range(12)])
    delta = np.zeros_like(theta)
    delta[3:5, 3:5, 3:5] = 1.0
    h = 0.2
    s2 = oracle.Scene(cam, theta - h * delta, theta + h * delta, albedo_const=0.8, max_depth=6, envmap=env)
    est = []
    for seed in range(12):
        H, F = oracle.render_twostates(s2, seed=7 + seed, spp=64)
        est.append(float(((F.astype(np.float64) - H) * w).sum() / (2 * h)))
    fd, fd_se = np.mean(est), np.std(est) / np.sqrt(len(est))
    proj = (runs * delta).sum(axis=(1, 2, 3))
    adj, adj_se = proj.mean(), proj.std() / np.sqrt(len(proj))
    assert abs(fd - adj) < 4 * np.hypot(fd_se, adj_se) + 1e-4, (fd, fd_se, adj, adj_se)
    assert abs(adj) > 3 * adj_se


def test_envmap_volpathsimple_adjoint_and_primal(oracle):
    """volpathsimple under a peaked map: its primal image has the two-state
    tracer's expectation (other sampling), and its adjoint (NEE with map
    importance sampling and MIS, DRT, transmittance terms) matches central
    differences of the two-state tracer."""
    res, D = 12, 8
    cam = oracle.camera_basis(res, res)
    env = random_map()
    theta = scenes.blob_density(D, 4)[..., 0] * 0.5
    sc = oracle.Scene(cam, theta, theta, albedo_const=0.8, max_depth=6, envmap=env)
    a = np.stack([oracle.vps_render(sc, seed=s, spp=256) for s in range(6)]).astype(np.float64)
    b = np.stack([oracle.render(sc, seed=50 + s, spp=256) for s in range(6)]).astype(np.float64)
    ma, mb = a.mean(axis=(1, 2, 3)), b.mean(axis=(1, 2, 3))
    se = np.hypot(ma.std(ddof=1), mb.std(ddof=1)) / np.sqrt(6)
    assert abs(ma.mean() - mb.mean()) < 4 * se + 1e-4, (ma.mean(), mb.mean(), se)
    w = np.random.default_rng(0).normal(0, 1, (res, res, 3)).astype(np.float32) + 0.5
    runs = np.array([oracle.vps_backward(sc, seed=100 + s, spp=32, grad_img=w)[0] for s in range(16)])
    delta = theta / theta.max()
    h = 0.02
    s2 = oracle.Scene(cam, theta - h * delta, theta + h * delta, albedo_const=0.8, max_depth=6, envmap=env)
    est = []
    for seed in range(12):
        H, F = oracle.render_twostates(s2, seed=7 + seed, spp=64)
        est.append(float(((F.astype(np.float64) - H) * w).sum() / (2 * h)))
    fd, fd_se = np.mean(est), np.std(est) / np.sqrt(len(est))
    proj = (runs * delta).sum(axis=(1, 2, 3))
    adj, adj_se = proj.mean(), proj.std() / np.sqrt(len(proj))
    assert abs(fd - adj) < 4 * np.hypot(fd_se, adj_se) + 1e-4, (fd, fd_se, adj, adj_se)
    assert abs(fd) > 4 * fd_se


def test_envmap_plugin_on_the_host(tmp_path):
    from recursive_control_variates_gb300 import io

    env = random_map()
    e = rcv.load_dict({"type": "envmap", "data": env, "scale": 0.5}, device="cpu")
    assert (e.width, e.height, e.scale) == (24, 12, 0.5)
    fn = tmp_path / "sky.exr"
    io.write_exr(str(fn), env)
    e2 = rcv.load_dict({"type": "envmap", "filename": str(fn)}, device="cpu")
    assert torch.equal(e2.texels, torch.from_numpy(env))
    with pytest.raises(ValueError):
        rcv.load_dict({"type": "envmap", "data": -env}, device="cpu")
    d = scenes.scene_dict(scenes.blob_density(8, 0), 0.8, res=8)
    d["emitter"] = {"type": "envmap", "data": env}
    sc = rcv.load_dict(d, device="cpu")
    assert sc.envmap() is not None
    d["sky"] = {"type": "constant"}
    with pytest.raises(ValueError):
        rcv.load_dict(d, device="cpu").envmap()


# ------------------------------------------------------------------- GPU
def gpu_env_scene(cuda, env, scale, res=32, albedo_grid=True):
    old = scenes.blob_density(16, 1)
    new = scenes.blob_density(16, 2)
    ao = scenes.albedo_grid(16, 1) if albedo_grid else None
    an = scenes.albedo_grid(16, 2) if albedo_grid else None
    d = scenes.scene_dict(new, an if albedo_grid else 0.8, res=res)
    d["emitter"] = {"type": "envmap", "data": env, "scale": scale}
    scene = rcv.load_dict(d, device=cuda)
    med = scene.named_shapes()["object"].interior_medium()
    med.old.density.copy_(torch.from_numpy(old))
    if albedo_grid:
        med.old.albedo_grid.copy_(torch.from_numpy(ao))
    med._dirty = True
    return scene, (old, new, ao, an)


def oracle_env_scene(O, scene, grids, env, scale, max_depth=8, rr_depth=None):
    s = scene.sensors()[0].c_struct()
    cam = O.Camera(s.width, s.height, tuple(s.origin), tuple(s.forward), tuple(s.right), tuple(s.up))
    old, new, ao, an = grids
    return O.Scene(cam, old[..., 0], new[..., 0], albedo_old=ao, albedo_new=an, albedo_const=0.8, max_depth=max_depth,
                   rr_depth=max_depth if rr_depth is None else rr_depth, envmap=env, envmap_scale=scale)


def frac_equal(a, b):
    return float(np.mean(np.all(a == b, axis=-1)))


@pytest.mark.gpu
@pytest.mark.parametrize("max_depth,rr_depth", [(8, 8), (12, 3)])
def test_envmap_tracers_match_oracle(cuda, oracle, max_depth, rr_depth):
    env, scale = random_map(), 1.7
    scene, grids = gpu_env_scene(cuda, env, scale)
    osc = oracle_env_scene(oracle, scene, grids, env, scale, max_depth, rr_depth)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": max_depth, "rr_depth": rr_depth})
    H, F = integ.render_twostates(scene, 0, seed=11, spp=8)
    S = integ.render(scene, 0, seed=12, spp=8)
    Ho, Fo = oracle.render_twostates(osc, seed=11, spp=8)
    So = oracle.render(osc, seed=12, spp=8)
    for name, a, b in (("H", H, Ho), ("F", F, Fo), ("single", S, So)):
        a = a.cpu().numpy()
        assert frac_equal(a, b) >= 0.999, name
        np.testing.assert_allclose(a.mean(), b.mean(), rtol=1e-5)
    # the map is not the constant environment
    plain = rcv.load_dict(scenes.scene_dict(grids[1], grids[3], res=32), device=cuda)
    assert not torch.equal(integ.render(plain, 0, seed=12, spp=8), S)
    params = rcv.traverse(scene)
    gimg = np.random.default_rng(4).normal(0, 1, (32, 32, 3)).astype(np.float32)
    grads = integ.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=13, spp=8)
    od, oa = oracle.backward(osc, seed=13, spp=8, grad_img=gimg)
    gd = grads[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    ga = grads[scenes.ALBEDO_KEY].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(gd - od) <= 2e-5 * np.linalg.norm(od)
    assert np.linalg.norm(ga - oa) <= 2e-5 * np.linalg.norm(oa)


@pytest.mark.gpu
def test_envmap_forward_mode_and_file(cuda, oracle, tmp_path):
    from recursive_control_variates_gb300 import io

    env, scale = random_map(seed=2), 0.9
    fn = tmp_path / "sky.exr"
    io.write_exr(str(fn), env)
    scene, grids = gpu_env_scene(cuda, env, scale, res=24)
    d = scenes.scene_dict(grids[1], grids[3], res=24)
    d["emitter"] = {"type": "envmap", "filename": str(fn), "scale": scale}
    scene_file = rcv.load_dict(d, device=cuda)
    med = scene_file.named_shapes()["object"].interior_medium()
    med.old.density.copy_(torch.from_numpy(grids[0]))
    med.old.albedo_grid.copy_(torch.from_numpy(grids[2]))
    med._dirty = True
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    assert torch.equal(integ.render(scene, 0, seed=3, spp=4), integ.render(scene_file, 0, seed=3, spp=4))
    params = rcv.traverse(scene)
    rng = np.random.default_rng(3)
    delta = rng.normal(0, 1, (16, 16, 16, 1)).astype(np.float32)
    fw = integ.render_forward(scene, params, 0, seed=5, spp=4,
                              tangents={scenes.DENSITY_KEY: torch.from_numpy(delta).to(cuda)})
    osc = oracle_env_scene(oracle, scene, grids, env, scale)
    ofw = oracle.forward(osc, seed=5, spp=4, tangent_density=delta[..., 0]).astype(np.float64)
    f = fw.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(ofw) > 0
    assert np.linalg.norm(f - ofw) <= 2e-5 * np.linalg.norm(ofw)


@pytest.mark.gpu
@pytest.mark.parametrize("flags", [{}, {"use_drt_subsampling": False}, {"use_nee": False}])
def test_envmap_volpathsimple_matches_oracle(cuda, oracle, flags):
    env, scale = random_map(seed=3), 1.3
    scene, grids = gpu_env_scene(cuda, env, scale, res=24)
    osc = oracle_env_scene(oracle, scene, grids, env, scale)
    vps = rcv.load_dict({"type": "volpathsimple", "max_depth": 8, "rr_depth": 8, **flags})
    img = vps.render(scene, 0, seed=3, spp=4).cpu().numpy()
    assert frac_equal(img, oracle.vps_render(osc, seed=3, spp=4, flags=flags)) >= 0.999
    params = rcv.traverse(scene)
    gimg = np.random.default_rng(5).normal(0, 1, (24, 24, 3)).astype(np.float32)
    g = vps.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=4, spp=4)
    od, oa = oracle.vps_backward(osc, seed=4, spp=4, grad_img=gimg, flags=flags)
    gd = g[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    ga = g[scenes.ALBEDO_KEY].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(gd - od) <= 2e-5 * np.linalg.norm(od)
    assert np.linalg.norm(ga - oa) <= 2e-5 * np.linalg.norm(oa)


@pytest.mark.gpu
def test_envmap_cv_step_and_rejections(cuda):
    """A cv step (two-state render, volpathsimple adjoint as in the grid
    experiments, experiments.py:131) under an envmap through the public API;
    the batched engine refuses the map."""
    env = random_map()
    scene, grids = gpu_env_scene(cuda, env, 1.0, res=24, albedo_grid=False)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath", "max_depth": 8},
                           "adjoint_integrator": {"type": "volpathsimple", "max_depth": 8}})
    opt = rcv.ad.Adam(lr=0.02)
    opt[scenes.DENSITY_KEY] = params[scenes.DENSITY_KEY]
    params.update(opt)
    target = torch.full((24, 24, 3), 0.5, device=cuda)
    for it in range(3):
        params.update(opt)
        img = rcv.render(scene, params, integrator=integ, seed=it, spp=4)
        loss = rcv.l2_loss(img, target)
        loss.backward()
        assert torch.isfinite(opt[scenes.DENSITY_KEY].grad).all()
        opt.step()
    assert np.isfinite(loss.item())
    from recursive_control_variates_gb300 import batch

    with pytest.raises(ValueError, match="constant environment"):
        batch.CVJob.from_scene(scene, params, integ, opt, target, spp=4)
