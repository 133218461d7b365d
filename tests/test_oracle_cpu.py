"""CPU checks of the oracle itself: known-answer vectors, golden fixtures made
by running the reference's own control-variate code, closed forms and
finite-difference consistency of its adjoint."""
import numpy as np
import pytest

from recursive_control_variates_gb300.scenes import blob_density


def test_pcg32_known_answer(oracle):
    # pcg32_srandom_r(42, 54): first outputs of O'Neill's reference demo
    expect = [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E]
    assert [int(v) for v in oracle.pcg32(42, 54, 6)] == expect


def test_tea_matches_library(oracle, rcvlib):
    from recursive_control_variates_gb300 import _lib

    rng = np.random.default_rng(1)
    for v0, v1 in rng.integers(0, 2**32, size=(200, 2), dtype=np.uint64):
        assert oracle.sample_tea_32(int(v0), int(v1)) == _lib.sample_tea_32(int(v0), int(v1))[0]


def test_uniform_stream_range(oracle):
    u = np.concatenate([oracle.rng_stream(7, lane, 64) for lane in range(64)])
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01
    # 23-bit grid
    assert np.all((u * 2**23) == np.floor(u * 2**23))


def test_log_accuracy(oracle):
    rng = np.random.default_rng(2)
    x = np.concatenate([rng.uniform(0, 1, 200000), 2.0 ** -np.arange(0, 24), [1.0]]).astype(np.float32)
    x = x[x > 0]
    got = oracle.log_unit(x).astype(np.float64)
    ref = np.log(x.astype(np.float64))
    err = np.abs(got - ref)
    assert np.all(err <= 2.5e-7 * np.maximum(1.0, np.abs(ref)))


def test_uniform_sphere(oracle):
    rng = np.random.default_rng(3)
    u = rng.uniform(0, 1, (50000, 2)).astype(np.float32)
    d = oracle.uniform_sphere(u).astype(np.float64)
    assert np.all(np.abs(np.linalg.norm(d, axis=1) - 1.0) < 2e-6)
    assert np.all(np.abs(d.mean(axis=0)) < 0.02)
    # azimuth follows the first sample, z the second
    np.testing.assert_allclose(d[:, 2], 1.0 - 2.0 * u[:, 1].astype(np.float64), atol=1e-6)
    phi = np.arctan2(d[:, 1], d[:, 0]) % (2 * np.pi)
    dphi = np.abs(phi - 2 * np.pi * u[:, 0])
    dphi = np.minimum(dphi, 2 * np.pi - dphi)
    assert np.all(dphi[np.linalg.norm(d[:, :2], axis=1) > 1e-3] < 2e-5)


def _scene(oracle, res=24, D=16, seeds=(1, 1), albedo=None, max_depth=8, rr_depth=None):
    cam = oracle.camera_basis(res, res)
    old = blob_density(D, seeds[0])
    new = blob_density(D, seeds[1])
    kw = {}
    if albedo is not None:
        kw = dict(albedo_old=albedo[0], albedo_new=albedo[1])
    return oracle.Scene(cam, old, new, max_depth=max_depth, rr_depth=rr_depth, **kw)


def test_two_state_equal_states_bitwise(oracle):
    """old == new: the two-state weights are exactly 1 and H == F == single
    (plugins/twostatevolpath.py:230-231, 259-260)."""
    sc = _scene(oracle)
    H, F = oracle.render_twostates(sc, seed=5, spp=8)
    S = oracle.render(sc, seed=5, spp=8)
    assert np.array_equal(H, F)
    assert np.array_equal(F, S)
    assert F.mean() > 0.05


def test_chunking_changes_only_summation_order(oracle):
    sc = _scene(oracle, seeds=(1, 2))
    H1, F1 = oracle.render_twostates(sc, seed=9, spp=8, chunk=8)
    H2, F2 = oracle.render_twostates(sc, seed=9, spp=8, chunk=1)
    np.testing.assert_allclose(F1, F2, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(H1, H2, rtol=1e-6, atol=1e-7)


def test_closed_form_transmittance(oracle):
    """Albedo 0, constant density: a pixel's expectation is the footprint
    average of exp(-sigma * chord)."""
    res, sigma = 16, 3.0
    cam = oracle.camera_basis(res, res)
    dens = np.full((8, 8, 8), sigma, np.float32)
    sc = oracle.Scene(cam, dens, dens, albedo_const=0.0, max_depth=16)
    spp = 1024
    img = oracle.render(sc, seed=3, spp=spp)[..., 0].astype(np.float64)
    o, f, r, u = (np.array(v, np.float64) for v in (cam.origin, cam.forward, cam.right, cam.up))
    sub = (np.arange(16) + 0.5) / 16
    expect = np.zeros((res, res))
    for py in range(res):
        for px in range(res):
            fx = px + sub[None, :]
            fy = py + sub[:, None]
            a = 2 * fx / res - 1
            b = 1 - 2 * fy / res
            d = f[None, None] + a[..., None] * r + b[..., None] * u
            d = d / np.linalg.norm(d, axis=-1, keepdims=True)
            with np.errstate(divide="ignore", invalid="ignore"):
                t0 = (0 - o) / d
                t1 = (1 - o) / d
            tn = np.max(np.minimum(t0, t1), -1)
            tf = np.min(np.maximum(t0, t1), -1)
            chord = np.where(tn <= tf, np.maximum(tf - np.maximum(tn, 0), 0), 0)
            expect[py, px] = np.exp(-sigma * chord).mean()
    sd = np.sqrt(np.maximum(expect * (1 - expect), 1e-4) / spp)
    z = np.abs(img - expect) / sd
    assert np.mean(z < 3) > 0.98
    assert abs(img.mean() - expect.mean()) < 4 * np.sqrt((sd**2).sum()) / img.size + 2e-3


def _footprint_transmittance(cam, px0, res_w, res_h, sigma, box_min, box_size, sub=8):
    """Footprint averages of exp(-sigma * chord) over the pixels of one
    sub-sensor, chords through the world box [box_min, box_min + box_size]."""
    o, f, r, u = (np.array(v, np.float64) for v in (cam.origin, cam.forward, cam.right, cam.up))
    lo = np.array(box_min, np.float64)
    hi = lo + np.array(box_size, np.float64)
    s = (np.arange(sub) + 0.5) / sub
    out = np.zeros((res_h, res_w))
    for py in range(res_h):
        for px in range(res_w):
            a = 2 * (px + s[None, :]) / res_w - 1
            b = 1 - 2 * (py + s[:, None]) / res_h
            d = f + a[..., None] * r + b[..., None] * u
            d = d / np.linalg.norm(d, axis=-1, keepdims=True)
            with np.errstate(divide="ignore", invalid="ignore"):
                t0 = (lo - o) / d
                t1 = (hi - o) / d
            tn = np.max(np.minimum(t0, t1), -1)
            tf = np.min(np.maximum(t0, t1), -1)
            chord = np.where(tn <= tf, np.maximum(tf - np.maximum(tn, 0), 0), 0)
            out[py, px] = np.exp(-sigma * chord).mean()
    return out


def test_box_transform_and_batch_film_closed_form(oracle):
    """Medium box to_world = translate * scale (experiments.py:57,64,79,285)
    and a batch film of 3 sub-sensors around it (experiments.py:28-50): with
    albedo 0 and constant density every sub-image is the footprint average of
    exp(-sigma * world chord) seen by its own sub-sensor."""
    w, h, sigma = 10, 8, 1.5
    box_min, box_size = (-0.3, 0.1, 0.2), (1.0, 1.2, 1.5)
    centre = np.array(box_min) + 0.5 * np.array(box_size)
    cams = []
    for k in range(3):
        th = 2 * np.pi * k / 3 + 0.1
        origin = centre + np.array([2.6 * np.cos(th), 0.4, 2.6 * np.sin(th)])
        cams.append(oracle.camera_basis(w, h, origin=tuple(origin), target=tuple(centre), up=(0, 1, 0), fov=45))
    dens = np.full((6, 5, 4), sigma, np.float32)  # non-cubic grid, constant
    sc = oracle.Scene(cams, dens, dens, albedo_const=0.0, max_depth=16, box_min=box_min, box_size=box_size)
    assert (sc.width, sc.height) == (3 * w, h)
    spp = 512
    img = oracle.render(sc, seed=5, spp=spp)[..., 0].astype(np.float64)
    for k in range(3):
        expect = _footprint_transmittance(cams[k], 0, w, h, sigma, box_min, box_size, sub=24)
        got = img[:, k * w:(k + 1) * w]
        # Bernoulli noise of the estimate plus the footprint quadrature error
        # at silhouette pixels
        sd = np.sqrt(np.maximum(expect * (1 - expect), 1e-4) / spp) + 0.004
        z = np.abs(got - expect) / sd
        assert np.mean(z < 3.5) > 0.95, (k, z.max())
        assert abs(got.mean() - expect.mean()) < 4 * np.sqrt((sd**2).sum()) / got.size + 2e-3
        assert expect.min() < 0.6  # the box is in view of every sub-sensor
    # the single-state and two-state tracers and volpathsimple agree
    H, F = oracle.render_twostates(sc, seed=5, spp=spp)
    assert np.array_equal(H, F) and np.array_equal(F[..., 0].astype(np.float64), img)
    v = oracle.vps_render(sc, seed=6, spp=spp)[..., 0].astype(np.float64)
    assert abs(v.mean() - img.mean()) < 0.01


def test_albedo_grid_with_own_resolution(oracle):
    """An albedo grid may have its own resolution (experiments.py:56,63:
    264x136x136 density, 256x128x128 albedo).  A constant grid at any
    resolution interpolates to exactly its value, so images and density
    gradients equal those of the constant albedo bit for bit, and the albedo
    gradients of two resolutions have the same total (up to the float
    rounding of the corner weights)."""
    cam = oracle.camera_basis(16, 16)
    old = blob_density(8, 1)
    new = blob_density(8, 2)
    plain = oracle.Scene(cam, old, new, albedo_const=0.8, max_depth=8)
    totals = []
    for res in [(5, 7, 9), (8, 8, 8), (16, 12, 3)]:
        a = np.full(res + (3,), 0.8, np.float32)
        sc = oracle.Scene(cam, old, new, albedo_old=a, albedo_new=a, max_depth=8)
        assert (sc.c.adz, sc.c.ady, sc.c.adx) == (res if res != (8, 8, 8) else (0, 0, 0))
        H, F = oracle.render_twostates(sc, seed=4, spp=4)
        Hp, Fp = oracle.render_twostates(plain, seed=4, spp=4)
        assert np.array_equal(H, Hp) and np.array_equal(F, Fp)
        g = np.random.default_rng(3).normal(0, 1, (16, 16, 3)).astype(np.float32)
        gd, ga = oracle.backward(sc, seed=9, spp=4, grad_img=g, threads=1)
        gdp, _ = oracle.backward(plain, seed=9, spp=4, grad_img=g, threads=1)
        assert np.array_equal(gd, gdp) and ga.shape == res + (3,)
        totals.append(ga.sum(axis=(0, 1, 2)))
        v = oracle.vps_render(sc, seed=2, spp=4)
        assert np.array_equal(v, oracle.vps_render(plain, seed=2, spp=4))
        _, va = oracle.vps_backward(sc, seed=5, spp=4, grad_img=g)
        assert va.shape == res + (3,)
    # the float corner weights of one event sum to 1 within a few ulp
    np.testing.assert_allclose(totals[0], totals[1], rtol=1e-6)
    np.testing.assert_allclose(totals[2], totals[1], rtol=1e-6)


def test_forward_mode_is_the_adjoint_transposed(oracle):
    """Forward mode (render_forward) and the adjoint replay the same paths
    and events: <w, J delta> equals <J^T w, delta> for the same seed, up to
    rounding; and the forward derivative matches central differences."""
    cam = oracle.camera_basis(16, 16)
    theta = blob_density(8, 4)[..., 0] * 0.5
    alb = np.full((8, 8, 8, 3), 0.6, np.float32) + 0.1 * np.random.default_rng(0).random((8, 8, 8, 3)).astype(np.float32)
    sc = oracle.Scene(cam, theta, theta, albedo_old=alb, albedo_new=alb, max_depth=6)
    rng = np.random.default_rng(1)
    w = rng.normal(0, 1, (16, 16, 3)).astype(np.float32)
    delta = rng.normal(0, 1, theta.shape).astype(np.float32)
    dalb = rng.normal(0, 1, alb.shape).astype(np.float32)
    fw = oracle.forward(sc, seed=21, spp=8, tangent_density=delta, tangent_albedo=dalb).astype(np.float64)
    gd, ga = oracle.backward(sc, seed=21, spp=8, grad_img=w)
    lhs = float((w.astype(np.float64) * fw).sum())
    rhs = float((gd * delta).sum() + (ga * dalb).sum())
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs)), (lhs, rhs)
    # statistical agreement with central differences (density only)
    delta = theta / theta.max()
    fws = [oracle.forward(sc, seed=100 + s, spp=32, tangent_density=delta).astype(np.float64) for s in range(12)]
    proj = np.array([(f * w).sum() for f in fws])
    h = 0.02
    s2 = oracle.Scene(cam, theta - h * delta, theta + h * delta, albedo_old=alb, albedo_new=alb, max_depth=6)
    est = []
    for seed in range(12):
        H, F = oracle.render_twostates(s2, seed=7 + seed, spp=64)
        est.append(float(((F.astype(np.float64) - H) * w).sum() / (2 * h)))
    fd, fd_sem = np.mean(est), np.std(est) / np.sqrt(len(est))
    fwd, fwd_sem = proj.mean(), proj.std() / np.sqrt(len(proj))
    assert abs(fd - fwd) < 4 * np.hypot(fd_sem, fwd_sem) + 1e-4, (fwd, fwd_sem, fd, fd_sem)


def test_cv_welford_golden(oracle, golden_cv):
    """The numpy restatement reproduces the reference's own CVIntegrator /
    MetaIntegrator / StatisticsEstimator code bit for bit."""
    g = golden_cv
    for name in g["cases"]:
        cv = oracle.CVOracle(
            warmup=int(g[f"{name}/warmup"]),
            beta1=float(g[f"{name}/beta1"]),
            beta2=float(g[f"{name}/beta2"]),
            pre_update=bool(g[f"{name}/pre_update"]),
        )
        H, F = g[f"{name}/H"], g[f"{name}/F"]
        for i in range(len(H)):
            with np.errstate(all="ignore"):
                img = cv.step(H[i], F[i])
            np.testing.assert_array_equal(np.broadcast_to(img, H[i].shape), g[f"{name}/img"][i], err_msg=str(name))
            np.testing.assert_array_equal(np.broadcast_to(cv.w_s, H[i].shape), g[f"{name}/w_s"][i])
            np.testing.assert_array_equal(np.broadcast_to(cv.stats.cov, H[i].shape), g[f"{name}/cov"][i])
            assert cv.stats.n == int(g[f"{name}/n"][i])


def _meta_feeds(g, name):
    """Nested-render callables over the recorded feeds of a meta case, with a
    call log of (kind, seed) like the generator's stub."""
    two = iter(g[f"{name}/twostate_feed"])
    single = iter(g[f"{name}/single_feed"])
    calls = []

    def render_twostates(seed):
        calls.append((0, int(seed)))
        hf = next(two)
        return hf[0], hf[1]

    def render(seed):
        calls.append((1, int(seed)))
        return next(single)

    return render_twostates, render, calls


def test_meta_cv_pss_and_force_baseline_golden(oracle, golden_cv):
    """MetaIntegrator's cv_pss (F = render(seed), H = the previous step's
    render(seed + 1), H = 0 at the first step), force_baseline and baseline
    returns: the numpy restatement reproduces the reference's own
    plugins/metaintegrator.py:57-130 bit for bit, with the same nested calls
    and seeds in the same order."""
    g = golden_cv
    for name in g["meta_cases"]:
        method = str(g[f"{name}/method"])
        m = oracle.MetaOracle(method, pre_update=bool(g[f"{name}/pre_update"]),
                              force_baseline=bool(g[f"{name}/force_baseline"]))
        r2, r1, calls = _meta_feeds(g, name)
        seed0 = int(g[f"{name}/seed0"])
        for i in range(len(g[f"{name}/out"])):
            with np.errstate(all="ignore"):
                out = m.render(r2, r1, seed0 + i)
            np.testing.assert_array_equal(out, g[f"{name}/out"][i], err_msg=f"{name} step {i}")
            np.testing.assert_array_equal(np.broadcast_to(m.img, out.shape), g[f"{name}/img"][i])
            if m.cv is not None:
                np.testing.assert_array_equal(np.broadcast_to(m.cv.w_s, out.shape), g[f"{name}/w_s"][i])
                np.testing.assert_array_equal(np.broadcast_to(m.cv.stats.cov, out.shape), g[f"{name}/cov"][i])
                assert m.cv.stats.n == int(g[f"{name}/n"][i])
        assert calls == [tuple(c) for c in g[f"{name}/calls"].tolist()], name
    # force_baseline returns the noisy (cv_pss) or a fresh single-state
    # (cv_ps) render while the control variate advances as without it
    for force, method in (("meta_cv_pss_force", "cv_pss"), ("meta_cv_ps_force", "cv_ps")):
        m = oracle.MetaOracle(method)
        r2, r1, _ = _meta_feeds(g, force)
        if method == "cv_ps":
            r1 = lambda seed: None  # noqa: E731  (no single-state render without force_baseline)
        for i in range(len(g[f"{force}/out"])):
            with np.errstate(all="ignore"):
                img = m.render(r2, r1, int(g[f"{force}/seed0"]) + i)
            np.testing.assert_array_equal(img, g[f"{force}/img"][i])
    np.testing.assert_array_equal(g["meta_cv_pss_force/out"], g["meta_cv_pss_force/single_feed"][0::2])
    np.testing.assert_array_equal(g["meta_cv_ps_force/out"], g["meta_cv_ps_force/single_feed"])
    assert not np.array_equal(g["meta_cv_ps_force/out"], g["meta_cv_ps_force/img"])


def test_steady_state_anchor(oracle):
    """Static scene, H == F (figures/steady_state/generate_data.py:56-79):
    the statistics of H and F are then bitwise equal, the control weight
    follows the analytic running-mean weight j/(j+1), and the image error
    falls like 1/j as the running mean's does (the recursion drops the
    first two renders and estimates its weights, so its error stays within
    a constant factor of the running mean's)."""
    rng = np.random.default_rng(5)
    n = 20000
    mu = rng.uniform(0.5, 1.5, n).astype(np.float32)
    cv = oracle.CVOracle()
    acc = np.zeros(n)
    mse = {}
    for j in range(40):
        F = (mu * rng.gamma(2.0, 0.5, n)).astype(np.float32)
        with np.errstate(all="ignore"):
            img = cv.step(F, F)
        np.testing.assert_array_equal(cv.stats.var_x, cv.stats.cov)
        np.testing.assert_array_equal(cv.stats.var_y, cv.stats.cov)
        acc += F
        mse[j] = (np.mean((img - mu) ** 2), np.mean((acc / (j + 1) - mu) ** 2))
        if j >= 5:
            if j >= 6:
                assert abs(float(np.median(cv.w_s)) - j / (j + 1)) < 0.03, j
            assert 0.9 < mse[j][0] / mse[j][1] < 2.0, (j, mse[j])
    assert mse[39][0] < 0.25 * mse[5][0]


def test_welford1_golden(oracle, golden_cv):
    g = golden_cv
    est = oracle.WelfordOracle()
    for i, x in enumerate(g["welford1/x"]):
        est.update(x)
        np.testing.assert_array_equal(est.mean, g["welford1/mean"][i])
        np.testing.assert_array_equal(est.var, g["welford1/var"][i])
        np.testing.assert_array_equal(est.get(), g["welford1/get"][i])


def test_adjoint_matches_two_state_finite_differences(oracle):
    """The path-replay adjoint against central differences of the expected
    image, estimated with the two-state tracer (old = theta - h e_v,
    new = theta + h e_v share random numbers, so F - H has low variance)."""
    res, D = 20, 8
    cam = oracle.camera_basis(res, res)
    theta = blob_density(D, 4)[..., 0] * 0.5
    rng = np.random.default_rng(0)
    dLdimg = rng.normal(0, 1, (res, res, 3)).astype(np.float32)
    sc = oracle.Scene(cam, theta, theta, albedo_const=0.8, max_depth=6)
    runs = np.array([oracle.backward(sc, seed=100 + s, spp=64, grad_img=dLdimg)[0] for s in range(16)])

    def fd_estimate(delta, h, n=12):
        s2 = oracle.Scene(cam, theta - h * delta, theta + h * delta, albedo_const=0.8, max_depth=6)
        est = []
        for seed in range(n):
            H, F = oracle.render_twostates(s2, seed=7 + seed, spp=64)
            est.append(float(((F.astype(np.float64) - H) * dLdimg).sum() / (2 * h)))
        return np.mean(est), np.std(est) / np.sqrt(n)

    def check(delta, h):
        proj = (runs * delta).sum(axis=(1, 2, 3))
        adj, adj_sem = proj.mean(), proj.std() / np.sqrt(len(proj))
        fd, fd_sem = fd_estimate(delta, h)
        assert abs(fd - adj) < 4 * np.hypot(adj_sem, fd_sem) + 1e-4, (adj, adj_sem, fd, fd_sem)

    # density-weighted direction: path replay's 1/sigma_t terms are heavy
    # tailed in near-empty voxels, so weight the perturbation by the density
    check(theta / theta.max(), 0.02)
    # single voxels where the medium is dense
    for flat in np.argsort(-theta.ravel())[:3]:
        delta = np.zeros_like(theta)
        delta[np.unravel_index(flat, theta.shape)] = 1.0
        check(delta, 0.05)


# ------------------------------------------------------- majorant supergrid
def _sg_scene(O, factor, D=16, res=12, depth=8):
    cam = O.camera_basis(res, res)
    dens = blob_density(D, 11)[..., 0]
    dens_old = blob_density(D, 12)[..., 0]
    return O.Scene(cam, dens_old, dens, albedo_const=0.8, max_depth=depth, majorant_factor=factor)


def _mean_images(O, scene, fn, seeds, spp, counters=None):
    outs = [fn(scene, seed=s, spp=spp, counters=counters) for s in seeds]
    return outs


@pytest.mark.parametrize("factor", [3, 4, 16])
def test_supergrid_render_is_unbiased(oracle, factor):
    """A majorant supergrid (DDA free-flight sampling, plugins/twostatemedium.py:25-70)
    changes which null collisions are sampled, not the expectation: image
    means agree with the global-majorant ones within noise (4 x 144 px x 128
    spp each: < 2.5 % relative, about 5 sigma), and sparse media need fewer
    density lookups."""
    g = _sg_scene(oracle, 0)
    s = _sg_scene(oracle, factor)
    cg, cs = np.zeros(4, np.uint64), np.zeros(4, np.uint64)
    rg = [oracle.render_twostates(g, seed=5 + k, spp=128, counters=cg) for k in range(4)]
    rs = [oracle.render_twostates(s, seed=5 + k, spp=128, counters=cs) for k in range(4)]
    for idx in (0, 1):  # H (old), F (new)
        mg = np.mean([r[idx].astype(np.float64).mean() for r in rg])
        ms = np.mean([r[idx].astype(np.float64).mean() for r in rs])
        assert abs(mg - ms) < 0.025 * mg, (idx, mg, ms)
    assert not np.array_equal(rg[0][1], rs[0][1])
    if factor < 16:
        assert cs[1] + cs[2] < cg[1] + cg[2]  # fewer lookups than the global majorant


def test_supergrid_single_state_and_adjoint_unbiased(oracle):
    g = _sg_scene(oracle, 0)
    s = _sg_scene(oracle, 4)
    a = np.mean([oracle.render(g, seed=2 + k, spp=128).mean() for k in range(4)])
    b = np.mean([oracle.render(s, seed=2 + k, spp=128).mean() for k in range(4)])
    assert abs(a - b) < 0.025 * a
    # d(mean image)/d(total density) of both estimators agree within noise
    dl = np.ones((12, 12, 3), np.float32)
    ta = np.array([oracle.backward(g, seed=40 + k, spp=64, grad_img=dl)[0].sum() for k in range(16)])
    tb = np.array([oracle.backward(s, seed=40 + k, spp=64, grad_img=dl)[0].sum() for k in range(16)])
    se = np.hypot(ta.std(ddof=1), tb.std(ddof=1)) / np.sqrt(16)
    assert abs(ta.mean() - tb.mean()) < 4 * se, (ta.mean(), tb.mean(), se)
    # not vacuous: denser media darken the image in most seeds (the estimates
    # are heavy-tailed through 1/sigma_n, so the sign, not the spread, is used)
    assert np.mean(ta < 0) >= 0.75 and np.mean(tb < 0) >= 0.75


# ------------------------------------------------------------ volpathsimple
def test_exp_nonpos_accuracy(oracle):
    xs = np.float32(-np.linspace(0.0, 86.9, 4001))
    got = np.array([oracle.exp_nonpos(float(x)) for x in xs], np.float64)
    ref = np.exp(xs.astype(np.float64))
    assert np.max(np.abs(got - ref) / ref) < 2.0 ** -23
    assert oracle.exp_nonpos(0.0) == 1.0 and oracle.exp_nonpos(-100.0) == 0.0


def test_vps_alt_seed_definition(oracle):
    """Second stream of the adjoint: sample_tea_32(bits of lane 0's seeding
    draw, 1)[0] (plugins/volpathsimple.py:108-113); the seeding draw is the
    fourth number of lane 0's stream (film 2D, channel 1D)."""
    for seed in (0, 7, 12345):
        u = oracle.rng_stream(seed, 0, 4)[3]
        bits = int(np.float32(u).view(np.uint32))
        assert oracle.vps_alt_seed(seed) == oracle.sample_tea_32(bits, 1)


def _vps_scene(O, albedo=0.8, D=8, res=20, depth=6, factor=0):
    cam = O.camera_basis(res, res)
    theta = blob_density(D, 4)[..., 0] * 0.5
    alb = albedo if np.isscalar(albedo) else albedo
    return O.Scene(cam, theta, theta, albedo_old=None if np.isscalar(alb) else alb,
                   albedo_new=None if np.isscalar(alb) else alb, albedo_const=0.8, max_depth=depth,
                   majorant_factor=factor), theta, cam


@pytest.mark.parametrize("factor", [0, 4])
def test_vps_primal_unbiased(oracle, factor):
    """volpathsimple renders the image of the single-state estimator (both
    estimate the same radiance): means within 2 %."""
    sc, theta, cam = _vps_scene(oracle, factor=factor)
    a = np.mean([oracle.render(sc, seed=s, spp=64).astype(np.float64).mean() for s in range(8)])
    b = np.mean([oracle.vps_render(sc, seed=s, spp=64).astype(np.float64).mean() for s in range(8)])
    assert abs(a - b) < 0.02 * a, (a, b)
    nn = oracle.vps_render(sc, seed=3, spp=64, flags={"use_nee": False})
    assert abs(float(nn.mean()) - a) < 0.05 * a


@pytest.mark.parametrize("flags", [{}, {"use_drt": False}, {"use_drt_subsampling": False},
                                   {"use_drt_mis": False}, {"use_nee": False}])
def test_vps_adjoint_matches_finite_differences(oracle, flags):
    """The volpathsimple adjoint (DRT scattering term, 4-sample transmittance
    term, NEE replay; plugins/volpathsimple.py:160-620) against central
    differences estimated with the two-state tracer (old = theta - h delta,
    new = theta + h delta share random numbers)."""
    sc, theta, cam = _vps_scene(oracle)
    res = sc.width
    rng = np.random.default_rng(0)
    dLdimg = rng.normal(0, 1, (res, res, 3)).astype(np.float32) + 0.5
    runs = np.array([oracle.vps_backward(sc, seed=100 + s, spp=32, grad_img=dLdimg, flags=flags)[0]
                     for s in range(24)])
    delta = theta / theta.max()
    h = 0.02
    s2 = oracle.Scene(cam, theta - h * delta, theta + h * delta, albedo_const=0.8, max_depth=6)
    est = []
    for seed in range(12):
        H, F = oracle.render_twostates(s2, seed=7 + seed, spp=64)
        est.append(float(((F.astype(np.float64) - H) * dLdimg).sum() / (2 * h)))
    fd, fd_sem = np.mean(est), np.std(est) / np.sqrt(len(est))
    proj = (runs * delta).sum(axis=(1, 2, 3))
    adj, adj_sem = proj.mean(), proj.std() / np.sqrt(len(proj))
    assert abs(fd - adj) < 4 * np.hypot(adj_sem, fd_sem) + 1e-4, (adj, adj_sem, fd, fd_sem)
    assert abs(fd) > 4 * fd_sem  # the check is not vacuous


def test_vps_albedo_gradient_matches_finite_differences(oracle):
    """Albedo-grid gradient of volpathsimple against central differences of
    the two-state tracer with old/new albedo = a -+ h."""
    D, res = 8, 20
    cam = oracle.camera_basis(res, res)
    theta = blob_density(D, 4)[..., 0] * 0.5
    alb = np.full((D, D, D, 3), 0.6, np.float32)
    sc = oracle.Scene(cam, theta, theta, albedo_old=alb, albedo_new=alb, max_depth=6)
    dLdimg = np.ones((res, res, 3), np.float32)
    runs = np.array([oracle.vps_backward(sc, seed=200 + s, spp=32, grad_img=dLdimg)[1] for s in range(16)])
    h = 0.05
    delta = np.zeros_like(alb)
    delta[..., 1] = 1.0  # green channel everywhere
    s2 = oracle.Scene(cam, theta, theta, albedo_old=alb - h * delta, albedo_new=alb + h * delta, max_depth=6)
    est = []
    for seed in range(12):
        H, F = oracle.render_twostates(s2, seed=9 + seed, spp=64)
        est.append(float(((F.astype(np.float64) - H) * dLdimg).sum() / (2 * h)))
    fd, fd_sem = np.mean(est), np.std(est) / np.sqrt(len(est))
    proj = (runs * delta).sum(axis=(1, 2, 3, 4))
    adj, adj_sem = proj.mean(), proj.std() / np.sqrt(len(proj))
    assert abs(fd - adj) < 4 * np.hypot(adj_sem, fd_sem) + 1e-4, (adj, adj_sem, fd, fd_sem)
    assert fd > 4 * fd_sem
