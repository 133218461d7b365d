"""GPU parity of the volumetric path: librcv kernels (through the C ABI)
against the CPU oracle on the same seeded inputs, plus statistical checks at
larger sizes.

Tolerances: tracers follow the same per-path float32 operation sequence as the
oracle, so pixel values are compared for exact equality on >= 99.9 % of pixels
(the remainder may differ where a path crosses a decision boundary within one
ulp); gradients accumulate with float atomics, compared at 2e-5 relative L2;
control-variate arithmetic within 1e-6 relative of the fixtures made by the
reference's own code."""
import ctypes as C

import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import _lib, scenes
from recursive_control_variates_gb300.utils import stream_handle

pytestmark = pytest.mark.gpu


def make_scene(device, D=16, res=40, seeds=(1, 2), albedo_grid=False, max_depth=8, spp=4):
    old = scenes.blob_density(D, seeds[0])
    new = scenes.blob_density(D, seeds[1])
    alb_old = scenes.albedo_grid(D, seeds[0]) if albedo_grid else None
    alb_new = scenes.albedo_grid(D, seeds[1]) if albedo_grid else None
    scene = rcv.load_dict(scenes.scene_dict(new, alb_new if albedo_grid else 0.8, res=res, spp=spp), device=device)
    med = scene.named_shapes()["object"].interior_medium()
    med.old.density.copy_(torch.from_numpy(old))
    if albedo_grid:
        med.old.albedo_grid.copy_(torch.from_numpy(alb_old))
    med._dirty = True
    return scene, med, (old, new, alb_old, alb_new)


def oracle_scene(O, scene, grids, max_depth, albedo_grid, majorant_factor=0):
    s = scene.sensors()[0].c_struct()
    cam = O.Camera(s.width, s.height, tuple(s.origin), tuple(s.forward), tuple(s.right), tuple(s.up))
    old, new, ao, an = grids
    return O.Scene(cam, old[..., 0], new[..., 0], albedo_old=ao, albedo_new=an, albedo_const=0.8,
                   max_depth=max_depth, rr_depth=max_depth, majorant_factor=majorant_factor)


def frac_equal(a, b):
    return np.mean(np.all(a == b, axis=-1))


@pytest.mark.parametrize("batch,blocks_per_sm,defer,order", [(1, 1, 1, "row_major"), (7, 2, 8, "longest_first"),
                                                             (64, 0, 32, "cost")])
@pytest.mark.parametrize("albedo_grid", [False, True])
def test_two_state_matches_oracle(cuda, oracle, batch, blocks_per_sm, defer, order, albedo_grid):
    """The persistent schedule (queue batch, resident blocks, deferral
    threshold, pixel hand-out order) changes which lane traces which path and
    when, never the result."""
    scene, med, grids = make_scene(cuda, albedo_grid=albedo_grid)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8, "batch": batch,
                           "blocks_per_sm": blocks_per_sm, "defer": defer, "order": order})
    H, F = integ.render_twostates(scene, 0, seed=11, spp=4)
    torch.cuda.synchronize()
    osc = oracle_scene(oracle, scene, grids, 8, albedo_grid)
    Ho, Fo = oracle.render_twostates(osc, seed=11, spp=4)
    H, F = H.cpu().numpy(), F.cpu().numpy()
    assert frac_equal(F, Fo) >= 0.999 and frac_equal(H, Ho) >= 0.999
    np.testing.assert_allclose(F.mean(), Fo.mean(), rtol=1e-5)
    np.testing.assert_allclose(H.mean(), Ho.mean(), rtol=1e-5)
    assert not np.array_equal(H, F)  # the states differ


def test_single_state_matches_oracle(cuda, oracle):
    scene, med, grids = make_scene(cuda)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    img = integ.render(scene, 0, seed=5, spp=8).cpu().numpy()
    ref = oracle.render(oracle_scene(oracle, scene, grids, 8, False), seed=5, spp=8)
    assert frac_equal(img, ref) >= 0.999


def test_equal_states_are_bitwise_identical(cuda):
    scene, med, grids = make_scene(cuda, seeds=(3, 3))
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    H, F = integ.render_twostates(scene, 0, seed=2, spp=8)
    S = integ.render(scene, 0, seed=2, spp=8)
    assert torch.equal(H, F) and torch.equal(F, S)


@pytest.mark.parametrize("albedo_grid", [False, True])
def test_adjoint_matches_oracle(cuda, oracle, albedo_grid):
    scene, med, grids = make_scene(cuda, albedo_grid=albedo_grid, res=32)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    rng = np.random.default_rng(4)
    gimg = rng.normal(0, 1, (32, 32, 3)).astype(np.float32)
    grads = integ.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=77, spp=4)
    gd = grads[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    od, oa = oracle.backward(oracle_scene(oracle, scene, grids, 8, albedo_grid), seed=77, spp=4, grad_img=gimg)
    assert np.linalg.norm(gd - od) <= 2e-5 * np.linalg.norm(od)
    if albedo_grid:
        ga = grads[scenes.ALBEDO_KEY].cpu().numpy().astype(np.float64)
        assert np.linalg.norm(ga - oa) <= 2e-5 * np.linalg.norm(oa)


def _cv_state(n, dev):
    bufs = [torch.zeros(n, device=dev) for _ in range(8)]
    s = _lib.CvState()
    for name, b in zip(("img", "w_s", "v_n", "mean_x", "mean_y", "var_x", "var_y", "cov"), bufs):
        setattr(s, name, b.data_ptr())
    return s, dict(zip(("img", "w_s", "v_n", "mean_x", "mean_y", "var_x", "var_y", "cov"), bufs))


def test_cv_step_matches_reference_fixtures(cuda, golden_cv, rcvlib):
    g = golden_cv
    for name in g["cases"]:
        H, F = g[f"{name}/H"], g[f"{name}/F"]
        n = H.shape[1]
        s, bufs = _cv_state(n, cuda)
        cnt = C.c_int32(0)
        for i in range(len(H)):
            h = torch.from_numpy(H[i]).to(cuda)
            f = torch.from_numpy(F[i]).to(cuda)
            rc = rcvlib.rcv_cv_step(C.byref(s), n, h.data_ptr(), f.data_ptr(), i, int(g[f"{name}/warmup"]),
                                    C.byref(cnt), float(g[f"{name}/beta1"]), float(g[f"{name}/beta2"]),
                                    int(g[f"{name}/pre_update"]), stream_handle(cuda))
            _lib.check(rc)
            for key in ("img", "w_s", "v_n", "var_x", "var_y", "cov", "mean_x", "mean_y"):
                got = bufs[key].cpu().numpy()
                ref = g[f"{name}/{key}"][i]
                np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-30, err_msg=f"{name}/{key} step {i}")
            assert cnt.value == int(g[f"{name}/n"][i])


def test_meta_integrator_methods_match_reference_fixtures(cuda, golden_cv):
    """MetaIntegrator ``cv_pss`` (H = the previous step's render with seed + 1,
    zero at the first step), ``pre_update``, ``force_baseline`` (noisy image
    for cv_pss, a fresh single-state render for cv_ps, the control variate
    still advancing) and ``baseline``, driven with the nested renders recorded
    from the reference's own plugins/metaintegrator.py:57-130: images and
    statistics within 1e-6 relative, the same nested calls with the same
    seeds in the same order."""
    g = golden_cv
    for name in g["meta_cases"]:
        nested = rcv.load_dict({"type": "twostateprbvolpath"})
        two = iter(g[f"{name}/twostate_feed"])
        single = iter(g[f"{name}/single_feed"])
        calls = []

        def render_twostates(scene, sensor, seed, spp, _two=two, _calls=calls):
            _calls.append((0, int(seed)))
            hf = next(_two)
            return torch.from_numpy(hf[0]).to(cuda), torch.from_numpy(hf[1]).to(cuda)

        def render(scene, sensor, seed, spp, develop=True, evaluate=True, _single=single, _calls=calls):
            _calls.append((1, int(seed)))
            return torch.from_numpy(next(_single)).to(cuda)

        nested.render_twostates = render_twostates  # instance overrides keep the two-state type
        nested.render = render
        meta = rcv.load_dict({"type": "meta", "method": str(g[f"{name}/method"]), "integrator": nested,
                              "pre_update": bool(g[f"{name}/pre_update"]),
                              "force_baseline": bool(g[f"{name}/force_baseline"])})
        seed0 = int(g[f"{name}/seed0"])
        for i in range(len(g[f"{name}/out"])):
            out = meta.render(None, 0, seed0 + i, 4)
            np.testing.assert_allclose(out.cpu().numpy(), g[f"{name}/out"][i], rtol=1e-6, atol=1e-30,
                                       err_msg=f"{name} step {i}")
            np.testing.assert_allclose(meta.img.cpu().numpy(), g[f"{name}/img"][i], rtol=1e-6, atol=1e-30)
            if "cv" in str(g[f"{name}/method"]):
                np.testing.assert_allclose(meta.cv.w_s.cpu().numpy(), g[f"{name}/w_s"][i], rtol=1e-6, atol=1e-30)
                np.testing.assert_allclose(meta.cv.v_n.cpu().numpy(), g[f"{name}/v_n"][i], rtol=1e-6, atol=1e-30)
                np.testing.assert_allclose(meta.cv.stats.cov.cpu().numpy(), g[f"{name}/cov"][i], rtol=1e-6,
                                           atol=1e-30)
                assert meta.cv.stats.n == int(g[f"{name}/n"][i])
        assert calls == [tuple(c) for c in g[f"{name}/calls"].tolist()], name


def test_statistics_and_welford_estimators(cuda, golden_cv, oracle):
    from recursive_control_variates_gb300.plugins.welford import StatisticsEstimator, WelfordVarianceEstimator

    g = golden_cv
    est = WelfordVarianceEstimator(0.9, 0.999)
    for i, x in enumerate(g["welford1/x"]):
        est.update(torch.from_numpy(x).to(cuda))
        np.testing.assert_allclose(est.get().cpu().numpy(), g["welford1/get"][i], rtol=1e-6)
    H, F = g["cv_default/H"], g["cv_default/F"]
    st = StatisticsEstimator()
    so = oracle.StatisticsOracle()
    for i in range(len(H)):
        st.update(torch.from_numpy(H[i]).to(cuda), torch.from_numpy(F[i]).to(cuda))
        so.update(H[i], F[i])
        for a, b in zip(st.get(), so.get()):
            np.testing.assert_allclose(a.cpu().numpy(), b, rtol=1e-6)


def test_losses_and_adam(cuda, oracle):
    rng = np.random.default_rng(9)
    x = rng.normal(0, 1, (64, 48, 3)).astype(np.float32)
    y = rng.normal(0, 1, (64, 48, 3)).astype(np.float32)
    X = torch.from_numpy(x).to(cuda).requires_grad_(True)
    Y = torch.from_numpy(y).to(cuda)
    l2 = rcv.l2_loss(X, Y)
    l2.backward()
    ref = np.mean((x.astype(np.float64) - y) ** 2)
    np.testing.assert_allclose(l2.item(), ref, rtol=1e-6)
    np.testing.assert_allclose(X.grad.cpu().numpy(), 2 * (x - y) / x.size, rtol=1e-6, atol=1e-12)
    l1 = rcv.l1_loss(X.detach(), Y)
    np.testing.assert_allclose(l1.item(), np.mean(np.abs(x.astype(np.float64) - y)), rtol=1e-6)
    # Adam + clamp against the numpy restatement
    p = rng.uniform(0, 2, 1000).astype(np.float32)
    opt = rcv.ad.Adam(lr=0.05)
    opt["p"] = p
    opt.set_bounds("p", 0.0, 1.5)
    pn, m, v = p.copy(), np.zeros_like(p), np.zeros_like(p)
    for t in range(1, 6):
        gr = rng.normal(0, 1, 1000).astype(np.float32)
        opt["p"].grad = torch.from_numpy(gr).to(cuda)
        opt.step()
        pn, m, v = oracle.adam_step(pn, gr, m, v, t, 0.05, lo=0.0, hi=1.5)
        np.testing.assert_allclose(opt["p"].detach().cpu().numpy(), pn, rtol=2e-6, atol=1e-7)
        assert float(opt["p"].grad.abs().max()) == 0.0


def _oracle_scene_opts(O, scene, grids, max_depth, rr_depth, hide, albedo_grid=True):
    s = scene.sensors()[0].c_struct()
    cam = O.Camera(s.width, s.height, tuple(s.origin), tuple(s.forward), tuple(s.right), tuple(s.up))
    old, new, ao, an = grids
    return O.Scene(cam, old[..., 0], new[..., 0], albedo_old=ao if albedo_grid else None,
                   albedo_new=an if albedo_grid else None, albedo_const=0.8, max_depth=max_depth,
                   rr_depth=rr_depth, hide_emitters=hide)


@pytest.mark.parametrize("max_depth,rr_depth,hide", [(16, 2, False), (0, 0, False), (2, 1, True), (-1, 3, False)])
def test_depth_roulette_and_emitter_options_match_oracle(cuda, oracle, max_depth, rr_depth, hide):
    """Russian roulette below max_depth (the plugins' default is max_depth 6,
    rr_depth 5), max_depth 0 and 2, unlimited depth (-1, ended by the
    roulette) and hidden emitters: two-state, single-state and adjoint
    against the oracle.  The cooperative walk of the last paths only runs
    below the roulette depth, so these cases also cover its hand-over."""
    scene, med, grids = make_scene(cuda, albedo_grid=True, res=32)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": max_depth, "rr_depth": rr_depth,
                           "hide_emitters": hide})
    H, F = integ.render_twostates(scene, 0, seed=21, spp=4)
    S = integ.render(scene, 0, seed=22, spp=4)
    osc = _oracle_scene_opts(oracle, scene, grids, max_depth, rr_depth, hide)
    Ho, Fo = oracle.render_twostates(osc, seed=21, spp=4)
    So = oracle.render(osc, seed=22, spp=4)
    H, F, S = H.cpu().numpy(), F.cpu().numpy(), S.cpu().numpy()
    for a, b in ((H, Ho), (F, Fo), (S, So)):
        assert frac_equal(a, b) >= 0.999
        np.testing.assert_allclose(a.mean(), b.mean(), rtol=1e-5)
    if hide:
        assert float(S.min()) == 0.0  # pixels whose rays miss the medium see nothing
    rng = np.random.default_rng(max_depth + 10)
    gimg = rng.normal(0, 1, (32, 32, 3)).astype(np.float32)
    grads = integ.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=23, spp=4)
    od, oa = oracle.backward(osc, seed=23, spp=4, grad_img=gimg)
    gd = grads[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    ga = grads[scenes.ALBEDO_KEY].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(od) > 0
    assert np.linalg.norm(gd - od) <= 2e-5 * np.linalg.norm(od)
    if np.linalg.norm(oa) > 0:
        assert np.linalg.norm(ga - oa) <= 2e-5 * np.linalg.norm(oa)
    else:
        assert float(np.abs(ga).max()) == 0.0  # max_depth 0: no scattering event


def test_empty_medium(cuda, oracle):
    """All-zero density (majorant 0): no collision, every path sees the
    environment (radiance 1) unattenuated, and no gradient event happens."""
    D = 8
    zero = np.zeros((D, D, D, 1), np.float32)
    scene = rcv.load_dict(scenes.scene_dict(zero, 0.8, res=16), device=cuda)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    H, F = integ.render_twostates(scene, 0, seed=3, spp=4)
    assert torch.equal(H, torch.ones_like(H)) and torch.equal(F, torch.ones_like(F))
    osc = _oracle_scene_opts(oracle, scene, (zero, zero, None, None), 8, 8, False, albedo_grid=False)
    Ho, Fo = oracle.render_twostates(osc, seed=3, spp=4)
    assert np.array_equal(F.cpu().numpy(), Fo) and np.array_equal(H.cpu().numpy(), Ho)
    g = integ.render_backward(scene, params, torch.ones((16, 16, 3), device=cuda), 0, seed=4, spp=4)
    assert float(g[scenes.DENSITY_KEY].abs().max()) == 0.0


def test_one_pixel_one_sample_matches_oracle(cuda, oracle):
    """A 1 x 1 film at spp 1: one path per launch (one warp, one lane)."""
    scene, med, grids = make_scene(cuda, res=1, albedo_grid=True)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 16, "rr_depth": 4})
    osc = _oracle_scene_opts(oracle, scene, grids, 16, 4, False)
    for seed in range(6):
        H, F = integ.render_twostates(scene, 0, seed=seed, spp=1)
        Ho, Fo = oracle.render_twostates(osc, seed=seed, spp=1)
        assert np.array_equal(H.cpu().numpy(), Ho) and np.array_equal(F.cpu().numpy(), Fo)
        grads = integ.render_backward(scene, params, torch.ones((1, 1, 3), device=cuda), 0, seed=seed, spp=1)
        od, _ = oracle.backward(osc, seed=seed, spp=1, grad_img=np.ones((1, 1, 3), np.float32))
        gd = grads[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
        assert np.linalg.norm(gd - od) <= 2e-5 * max(np.linalg.norm(od), 1e-30)


def test_autograd_render_matches_direct_backward(cuda):
    scene, med, grids = make_scene(cuda, seeds=(1, 1), res=24)
    params = rcv.traverse(scene)
    opt = rcv.ad.Adam(lr=0.01)
    opt[scenes.DENSITY_KEY] = params[scenes.DENSITY_KEY]
    params.update(opt)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    img = rcv.render(scene, params, integrator=integ, seed=4, spp=4, spp_grad=8)
    w = torch.randn_like(img)
    (img * w).sum().backward()
    direct = integ.render_backward(scene, params, w, 0, seed=rcv.default_seed_grad(4), spp=8)
    torch.testing.assert_close(opt[scenes.DENSITY_KEY].grad, direct[scenes.DENSITY_KEY], rtol=1e-4, atol=1e-6)


def test_adjoint_started_ahead_matches_full_adjoint(cuda):
    """The adjoint's radiance pass started on a side stream before the
    gradient is known (rcv_render_adjoint_radiance) plus the replay equals
    the one-call adjoint; a parameter change in between invalidates it."""
    scene, med, grids = make_scene(cuda, res=32, albedo_grid=True)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    g = torch.randn((32, 32, 3), device=cuda)
    full = integ.render_backward(scene, params, g, 0, seed=5, spp=4)
    assert integ.last_adjoint_call == "rcv_render_backward_volume"
    launch = integ.prefetch_adjoint(scene, 0, seed=5, spp=4)
    H, F = integ.render_twostates(scene, 0, seed=9, spp=4)  # primal work in between
    launch()
    split = integ.render_backward(scene, params, g, 0, seed=5, spp=4)
    assert integ.last_adjoint_call == "rcv_render_backward_replay"
    for key in (scenes.DENSITY_KEY, scenes.ALBEDO_KEY):
        a, b = full[key].double(), split[key].double()
        assert float((a - b).norm()) <= 2e-5 * float(a.norm())
    H2, F2 = integ.render_twostates(scene, 0, seed=9, spp=4)
    assert torch.equal(H, H2) and torch.equal(F, F2)
    assert int(integ.counters(cuda).abs().sum()) == 0  # event counting is off by default
    # stale: another seed, or the parameters changed after the radiance pass
    integ.prefetch_adjoint(scene, 0, seed=6, spp=4)()
    integ.render_backward(scene, params, g, 0, seed=7, spp=4)
    assert integ.last_adjoint_call == "rcv_render_backward_volume"
    integ.prefetch_adjoint(scene, 0, seed=5, spp=4)()
    med.new.density.mul_(1.01)
    med._dirty = True
    changed = integ.render_backward(scene, params, g, 0, seed=5, spp=4)
    assert integ.last_adjoint_call == "rcv_render_backward_volume"
    assert not torch.equal(changed[scenes.DENSITY_KEY], full[scenes.DENSITY_KEY])


def test_finite_differences_32_voxels(cuda):
    """Adjoint vs central differences (h = 1e-3) on 32 random voxels of a
    64^3 density + albedo grid (config-2 medium at 96^2), with the
    differences estimated by the two-state tracer (shared random numbers)."""
    D, res, depth = 64, 96, 16
    theta = scenes.blob_density(D, 0)
    alb = scenes.albedo_grid(D, 0)
    scene = rcv.load_dict(scenes.scene_dict(theta, alb, res=res), device=cuda)
    params = rcv.traverse(scene)
    med = scene.named_shapes()["object"].interior_medium()
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": depth, "rr_depth": depth})
    rng = np.random.default_rng(12)
    gimg = torch.from_numpy(rng.normal(0, 1, (res, res, 3)).astype(np.float32)).to(cuda)
    runs = []
    for s in range(8):
        runs.append(integ.render_backward(scene, params, gimg, 0, seed=1000 + s, spp=64)[scenes.DENSITY_KEY][..., 0])
    runs = torch.stack(runs).double()
    dens = theta[..., 0]
    cand = np.flatnonzero(dens.ravel() > 0.5 * dens.max())
    voxels = rng.choice(cand, 32, replace=False)
    h = 1e-3
    z = []
    base = torch.from_numpy(theta).to(cuda)
    for flat in voxels:
        v = np.unravel_index(flat, dens.shape)
        lo, hi = base.clone(), base.clone()
        lo[v] -= h
        hi[v] += h
        med.old.density.copy_(lo)
        med.new.density.copy_(hi)
        med._dirty = True
        est = []
        for s in range(8):
            H, F = integ.render_twostates(scene, 0, seed=50 + s, spp=64)
            est.append(float(((F.double() - H.double()) * gimg.double()).sum() / (2 * h)))
        fd, fd_sem = np.mean(est), np.std(est) / np.sqrt(len(est))
        a = runs[:, v[0], v[1], v[2]].cpu().numpy()
        adj, adj_sem = a.mean(), a.std() / np.sqrt(len(a))
        z.append((fd - adj) / max(np.hypot(fd_sem, adj_sem), 1e-12))
    z = np.abs(np.array(z))
    assert np.mean(z < 3.5) >= 0.9, z


def test_cv_optimisation_reduces_loss(cuda):
    cfg = scenes.CONFIGS["cfg1"]
    dens, alb = scenes.config_grids(cfg)
    scene_ref = rcv.load_dict(scenes.scene_dict(dens, alb, res=64), device=cuda)
    base = rcv.load_dict({"type": "prbvolpath", "max_depth": 16, "rr_depth": 16})
    target = base.render(scene_ref, 0, seed=17843, spp=256)
    init = np.full_like(dens, 1.0)
    scene = rcv.load_dict(scenes.scene_dict(init, alb, res=64), device=cuda)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath", "max_depth": 16, "rr_depth": 16}})
    opt = rcv.ad.Adam(lr=0.2)
    opt[scenes.DENSITY_KEY] = init
    opt.set_bounds(scenes.DENSITY_KEY, 0.0, 250.0)
    params.update(opt)
    params.update(opt)
    losses = []
    for it in range(30):
        params.update(opt)
        img = rcv.render(scene, params, integrator=integ, seed=it, spp=4)
        if it == 0:
            torch.testing.assert_close(img, integ.F)
        loss = rcv.l2_loss(img, target)
        loss.backward()
        opt.step()
        losses.append(loss.item())
    assert np.mean(losses[-5:]) < 0.7 * np.mean(losses[:3]), losses
    assert float(integ.w_s.max()) <= 1.0 and float(integ.w_s.min()) >= 0.0


def test_steady_state_anchor(cuda):
    """Static scene through the ``cv`` integrator (old == new, so H == F bit
    for bit), as figures/steady_state/generate_data.py:56-79 compares it:
    the statistics of H and F stay bitwise equal, the median control weight
    follows the analytic running-mean weight j/(j+1) (within 0.06 from step
    6 on, within 0.025 from step 20 on: the estimated weights lag behind it
    early), and the error of the image against a 4096-spp render falls like
    the running mean's (within a factor 0.8-2.5 of it, and by more than 4x
    from step 5 to step 39)."""
    cfg = scenes.CONFIGS["cfg1"]
    dens, alb = scenes.config_grids(cfg)
    res = 32
    scene = rcv.load_dict(scenes.scene_dict(dens, alb, res=res), device=cuda)
    base = rcv.load_dict({"type": "prbvolpath", "max_depth": cfg.max_depth, "rr_depth": cfg.max_depth})
    ref = base.render(scene, 0, seed=99991, spp=4096).double()
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath", "max_depth": cfg.max_depth,
                                                         "rr_depth": cfg.max_depth}})
    acc = torch.zeros_like(ref)
    mse, med = {}, {}
    for j in range(40):
        img = integ.render(scene, 0, seed=j, spp=4)
        assert torch.equal(integ.H, integ.F)
        st = integ.stats
        assert torch.equal(st.var_x, st.cov) and torch.equal(st.var_y, st.cov)
        acc += integ.F.double()
        mse[j] = (float(((img.double() - ref) ** 2).mean()), float(((acc / (j + 1) - ref) ** 2).mean()))
        if j >= 5:
            noisy = st.var_x > 1e-6 * float(st.var_x.max())
            med[j] = float(integ.w_s[noisy].median())
    dev = {j: round(m - j / (j + 1), 4) for j, m in med.items()}
    ratio = {j: round(mse[j][0] / mse[j][1], 3) for j in med}
    print("median weight - j/(j+1):", dev)
    print("image error / running-mean error:", ratio)
    assert all(abs(d) < 0.06 for j, d in dev.items() if j >= 6), dev
    assert all(abs(d) < 0.025 for j, d in dev.items() if j >= 20), dev
    assert all(0.8 < r < 2.5 for r in ratio.values()), ratio
    assert mse[39][0] < 0.25 * mse[5][0], (mse[5], mse[39])


def test_cost_order_changes_schedule_not_results(cuda):
    """RCV_ORDER_COST sorts each call's pixels by the path lengths the previous
    call measured (kept in the workspace); repeated calls therefore run in
    different orders and must give bit-identical images and gradients."""
    scene, med, grids = make_scene(cuda, albedo_grid=True)
    by_cost = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8, "order": "cost"})
    rows = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8, "order": "row_major"})
    ref_H, ref_F = rows.render_twostates(scene, 0, seed=21, spp=4)
    for _ in range(3):
        H, F = by_cost.render_twostates(scene, 0, seed=21, spp=4)
        assert torch.equal(H, ref_H) and torch.equal(F, ref_F)
    f = scene.sensors()[0].film()
    ws = by_cost._scratch[cuda]
    lib = _lib.load()
    L_order = 256 + 1024  # counter + buckets; the cost array follows the order array
    npix = f.width * f.height
    cost_off = ((L_order + npix * 4 + 255) // 256) * 256
    aligned = (ws.data_ptr() + 255) & ~255
    cost = ws[aligned - ws.data_ptr() + cost_off:][: npix * 4].view(torch.int32)
    assert int(cost.sum()) > 0  # the last call recorded its path lengths


@pytest.mark.parametrize("factor", [3, 8])
def test_supergrid_tracers_match_oracle(cuda, oracle, factor):
    """Majorant supergrid (plugins/twostatemedium.py:25-70): the DDA
    free-flight sampling of the two-state, single-state and adjoint kernels
    follows the oracle's float operations (images bit-identical on >= 99.9 %
    of pixels, gradients 2e-5), and it samples fewer collisions."""
    scene, med, grids = make_scene(cuda, albedo_grid=True, D=24, res=32)
    osc = oracle_scene(oracle, scene, grids, 8, True, factor)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8, "count_events": True})
    cnt_global = integ.counters(cuda).clone()
    integ.render_twostates(scene, 0, seed=3, spp=4)
    cnt_global = (integ.counters(cuda) - cnt_global).cpu().numpy()
    med.set_majorant_resolution_factor(factor)
    c0 = integ.counters(cuda).clone()
    H, F = integ.render_twostates(scene, 0, seed=3, spp=4)
    cnt_sg = (integ.counters(cuda) - c0).cpu().numpy()
    Ho, Fo = oracle.render_twostates(osc, seed=3, spp=4)
    H, F = H.cpu().numpy(), F.cpu().numpy()
    assert frac_equal(F, Fo) >= 0.999 and frac_equal(H, Ho) >= 0.999
    assert cnt_sg[1] + cnt_sg[2] < cnt_global[1] + cnt_global[2]
    img = integ.render(scene, 0, seed=9, spp=4).cpu().numpy()
    assert frac_equal(img, oracle.render(osc, seed=9, spp=4)) >= 0.999
    params = rcv.traverse(scene)
    gimg = np.random.default_rng(6).normal(0, 1, (32, 32, 3)).astype(np.float32)
    grads = integ.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=31, spp=4)
    od, oa = oracle.backward(osc, seed=31, spp=4, grad_img=gimg)
    gd = grads[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    ga = grads[scenes.ALBEDO_KEY].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(gd - od) <= 2e-5 * np.linalg.norm(od)
    assert np.linalg.norm(ga - oa) <= 2e-5 * np.linalg.norm(oa)


# ------------------------------------------- medium box and batch sensor
def box_batch_scene(device, seeds=(1, 2), albedo_grid=True, n_views=3, res=16, height=12, spp=4,
                    albedo_res=(12, 10, 8)):
    """The grid scenes' shape (experiments.py:28-80, 285): a non-cubic grid
    in a translated, scaled box seen by a batch of sub-sensors around it;
    ``albedo_res`` (Dz, Dy, Dx) may differ from the density's 12 x 10 x 8."""
    from recursive_control_variates_gb300.core import T

    box = T.translate([-0.3, 0.1, 0.2]).scale([1.0, 1.2, 1.5])
    old = np.ascontiguousarray(scenes.blob_density(12, seeds[0])[:, :10, :8])  # Dz, Dy, Dx = 12, 10, 8
    new = np.ascontiguousarray(scenes.blob_density(12, seeds[1])[:, :10, :8])
    az, ay, ax = albedo_res
    ao = np.ascontiguousarray(scenes.albedo_grid(16, seeds[0])[:az, :ay, :ax]) if albedo_grid else None
    an = np.ascontiguousarray(scenes.albedo_grid(16, seeds[1])[:az, :ay, :ax]) if albedo_grid else None
    views = scenes.orbit_views(box, n_views, distance=2.6, height=0.4)
    d = scenes.scene_dict(new, an if albedo_grid else 0.8, res=res, height=height, spp=spp, box=box, views=views)
    scene = rcv.load_dict(d, device=device)
    med = scene.named_shapes()["object"].interior_medium()
    med.old.density.copy_(torch.from_numpy(old))
    if albedo_grid:
        med.old.albedo_grid.copy_(torch.from_numpy(ao))
    med._dirty = True
    return scene, med, (old, new, ao, an)


def oracle_box_scene(O, scene, med, grids, max_depth, majorant_factor=0):
    s = scene.sensors()[0].c_struct()
    n = max(1, s.count)
    w = s.width // n
    frames = [(s.origin, s.forward, s.right, s.up)] + [(f.origin, f.forward, f.right, f.up) for f in s.more[:n - 1]]
    cams = [O.Camera(w, s.height, *(tuple(v) for v in fr)) for fr in frames]
    m = med.c_struct()
    old, new, ao, an = grids
    return O.Scene(cams, old, new, albedo_old=ao, albedo_new=an, albedo_const=0.8, max_depth=max_depth,
                   rr_depth=max_depth, majorant_factor=majorant_factor, box_min=tuple(m.box_min),
                   box_size=tuple(m.box_size))


@pytest.mark.parametrize("factor", [0, 3])
def test_box_and_batch_film_match_oracle(cuda, oracle, factor):
    """Medium box (to_world = translate * scale) and a 3-sensor batch film:
    two-state, single-state and adjoint tracers against the oracle (images
    >= 99.9 % bit-identical, gradients 2e-5), with and without a supergrid."""
    scene, med, grids = box_batch_scene(cuda)
    med.set_majorant_resolution_factor(factor)
    osc = oracle_box_scene(oracle, scene, med, grids, 8, factor)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    H, F = integ.render_twostates(scene, 0, seed=13, spp=4)
    assert tuple(F.shape) == (12, 48, 3)
    Ho, Fo = oracle.render_twostates(osc, seed=13, spp=4)
    H, F = H.cpu().numpy(), F.cpu().numpy()
    assert frac_equal(F, Fo) >= 0.999 and frac_equal(H, Ho) >= 0.999
    assert F[:, :16].mean() != F[:, 16:32].mean()  # the sub-sensors see different views
    img = integ.render(scene, 0, seed=5, spp=4).cpu().numpy()
    assert frac_equal(img, oracle.render(osc, seed=5, spp=4)) >= 0.999
    params = rcv.traverse(scene)
    gimg = np.random.default_rng(8).normal(0, 1, (12, 48, 3)).astype(np.float32)
    grads = integ.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=21, spp=4)
    od, oa = oracle.backward(osc, seed=21, spp=4, grad_img=gimg)
    gd = grads[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    ga = grads[scenes.ALBEDO_KEY].cpu().numpy().astype(np.float64)
    assert gd.shape == (12, 10, 8)
    assert np.linalg.norm(gd - od) <= 2e-5 * np.linalg.norm(od)
    assert np.linalg.norm(ga - oa) <= 2e-5 * np.linalg.norm(oa)
    vps = rcv.load_dict({"type": "volpathsimple", "max_depth": 8, "rr_depth": 8})
    v = vps.render(scene, 0, seed=3, spp=4).cpu().numpy()
    assert frac_equal(v, oracle.vps_render(osc, seed=3, spp=4)) >= 0.999
    vg = vps.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=22, spp=4)
    vd = vg[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    ovd, _ = oracle.vps_backward(osc, seed=22, spp=4, grad_img=gimg)
    assert np.linalg.norm(vd - ovd) <= 2e-5 * np.linalg.norm(ovd)


def test_albedo_grid_with_own_resolution_matches_oracle(cuda, oracle):
    """Albedo grid at its own resolution (experiments.py:56,63): tracers,
    adjoint (albedo gradient on the albedo grid) and volpathsimple against
    the oracle."""
    scene, med, grids = box_batch_scene(cuda, albedo_res=(7, 9, 5))
    assert med.albedo_dims == (5, 9, 7) and med.dims == (8, 10, 12)
    osc = oracle_box_scene(oracle, scene, med, grids, 8)
    assert (osc.c.adx, osc.c.ady, osc.c.adz) == (5, 9, 7)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    H, F = integ.render_twostates(scene, 0, seed=31, spp=4)
    Ho, Fo = oracle.render_twostates(osc, seed=31, spp=4)
    assert frac_equal(F.cpu().numpy(), Fo) >= 0.999 and frac_equal(H.cpu().numpy(), Ho) >= 0.999
    params = rcv.traverse(scene)
    gimg = np.random.default_rng(9).normal(0, 1, (12, 48, 3)).astype(np.float32)
    grads = integ.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=32, spp=4)
    od, oa = oracle.backward(osc, seed=32, spp=4, grad_img=gimg)
    ga = grads[scenes.ALBEDO_KEY].cpu().numpy().astype(np.float64)
    assert ga.shape == (7, 9, 5, 3) == oa.shape
    gd = grads[scenes.DENSITY_KEY].cpu().numpy()[..., 0].astype(np.float64)
    assert np.linalg.norm(gd - od) <= 2e-5 * np.linalg.norm(od)
    assert np.linalg.norm(ga - oa) <= 2e-5 * np.linalg.norm(oa)
    vps = rcv.load_dict({"type": "volpathsimple", "max_depth": 8, "rr_depth": 8})
    vg = vps.render_backward(scene, params, torch.from_numpy(gimg).to(cuda), 0, seed=33, spp=4)
    _, ova = oracle.vps_backward(osc, seed=33, spp=4, grad_img=gimg)
    va = vg[scenes.ALBEDO_KEY].cpu().numpy().astype(np.float64)
    assert np.linalg.norm(va - ova) <= 2e-5 * np.linalg.norm(ova)


def test_batched_engine_with_box_and_batch_film(cuda):
    """A batched job built from a box + batch-sensor scene renders the same
    first-step images as the plain API (seed = seed_base)."""
    from recursive_control_variates_gb300 import batch

    scene, med, grids = box_batch_scene(cuda, seeds=(2, 2), albedo_grid=False)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath", "max_depth": 8,
                                                         "rr_depth": 8}})
    opt = rcv.ad.Adam(lr=0.02)
    opt[scenes.DENSITY_KEY] = med.new.density.detach().clone()
    params.update(opt)
    params.update(opt)
    target = torch.full((12, 48, 3), 0.5, device=cuda)
    job = batch.CVJob.from_scene(scene, params, integ, opt, target, spp=4, seed=17, keep_images=True)
    b = batch.BatchedCV([job])
    b.step()
    torch.cuda.synchronize()
    params.update(opt)
    img = rcv.render(scene, params, integrator=integ, seed=17, spp=4)
    H, F = job.primal_images()
    assert torch.equal(F, integ.cv.F) and torch.equal(H, integ.cv.H)
    assert torch.equal(job.image(), img.detach())
    b.close()


def test_upsampling_schedule_step(cuda):
    """utils.upsample mid-optimisation (optimize.py:135-136): the next step
    renders and differentiates the doubled grids (old = new after the
    rotation, CV state reset), and the adjoint matches the oracle on them."""
    scene, med, grids = make_scene(cuda, D=8, res=24, seeds=(3, 3))
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath", "max_depth": 8,
                                                         "rr_depth": 8}})
    opt = rcv.ad.Adam(lr=0.02)
    opt[scenes.DENSITY_KEY] = med.new.density.detach().clone()
    params.update(opt)
    params.update(opt)
    target = torch.full((24, 24, 3), 0.4, device=cuda)
    for it in range(2):
        params.update(opt)
        rcv.l2_loss(rcv.render(scene, params, integrator=integ, seed=it, spp=2), target).backward()
        opt.step()
    rcv.utils.upsample(scene, {"variables": {scenes.DENSITY_KEY: {}}}, opt, integ)
    params.update(opt)
    assert med.dims == (16, 16, 16) and not integ.init
    img = rcv.render(scene, params, integrator=integ, seed=5, spp=2)
    rcv.l2_loss(img, target).backward()
    g = opt[scenes.DENSITY_KEY].grad
    assert tuple(g.shape) == (16, 16, 16, 1) and torch.isfinite(g).all() and float(g.abs().sum()) > 0
    H, F = integ.integrator.render_twostates(scene, 0, seed=7, spp=2)
    assert torch.equal(H, F)  # old = new right after the upsampling


def test_forward_mode_matches_oracle_and_adjoint(cuda, oracle):
    """render_forward (plugins/cv_integrator.py:79-85): the image derivative
    along density and albedo tangents against the oracle (2e-5 relative L2)
    and against the adjoint of the same paths (<w, J t> = <J^T w, t>); and
    torch forward-mode AD through rcv.render."""
    from torch.autograd import forward_ad

    scene, med, grids = make_scene(cuda, res=24, albedo_grid=True)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8})
    rng = np.random.default_rng(3)
    delta = rng.normal(0, 1, (16, 16, 16, 1)).astype(np.float32)
    dalb = rng.normal(0, 1, (16, 16, 16, 3)).astype(np.float32)
    tan = {scenes.DENSITY_KEY: torch.from_numpy(delta).to(cuda), scenes.ALBEDO_KEY: torch.from_numpy(dalb).to(cuda)}
    fw = integ.render_forward(scene, params, 0, seed=13, spp=4, tangents=tan)
    osc = oracle_scene(oracle, scene, grids, 8, True)
    ofw = oracle.forward(osc, seed=13, spp=4, tangent_density=delta[..., 0], tangent_albedo=dalb).astype(np.float64)
    f = fw.cpu().numpy().astype(np.float64)
    assert np.linalg.norm(ofw) > 0
    assert np.linalg.norm(f - ofw) <= 2e-5 * np.linalg.norm(ofw)
    w = rng.normal(0, 1, (24, 24, 3)).astype(np.float32)
    g = integ.render_backward(scene, params, torch.from_numpy(w).to(cuda), 0, seed=13, spp=4)
    lhs = float((w.astype(np.float64) * f).sum())
    rhs = float((g[scenes.DENSITY_KEY].cpu().double().numpy() * delta).sum()
                + (g[scenes.ALBEDO_KEY].cpu().double().numpy() * dalb).sum())
    assert abs(lhs - rhs) <= 1e-4 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    # forward-mode AD: a dual density tensor through rcv.render
    with forward_ad.dual_level():
        primal = params[scenes.DENSITY_KEY].detach().clone()
        params[scenes.DENSITY_KEY] = forward_ad.make_dual(primal, tan[scenes.DENSITY_KEY])
        params.update()
        img = rcv.render(scene, params, integrator=integ, seed=5, spp=4)
        jvp = forward_ad.unpack_dual(img).tangent
    direct = integ.render_forward(scene, params, 0, seed=rcv.default_seed_grad(5), spp=4,
                                  tangents={scenes.DENSITY_KEY: tan[scenes.DENSITY_KEY]})
    assert jvp is not None
    assert float((jvp - direct).norm()) <= 1e-5 * float(direct.norm())
