"""Batched cv_ps steps (librcv rcv_batch_*, recursive_control_variates_gb300.batch).

CPU: the bias-correction tables reproduce the host arithmetic of rcv_cv_step /
rcv_adam_step; batch descriptions are validated on the host.

GPU: a job advanced in a batch matches the same job advanced through the
plain API (load_dict / traverse / render / l2_loss / backward / ad.Adam).
Tolerances: the two-state images, the control-variate image and dL/dimage of a
step are bit-identical (same per-path arithmetic, same reduction order); the
loss sum is accumulated with double atomics (1e-6 relative); gradients use
float atomics in both forms, so the Adam moments agree to 1e-5 relative L2,
and later steps drift apart at the level of atomic reordering (a first Adam
step maps a gradient to +-lr by its sign, so a voxel whose gradient is ~0 can
move either way): images after several steps agree to 1e-3 relative L2."""
import ctypes as C
import math

import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import _lib, batch, scenes, serve


# ------------------------------------------------------------------- CPU
@pytest.mark.parametrize("beta", [0.0, 0.5, 0.9, 0.999])
def test_cv_table_matches_host_arithmetic(rcvlib, beta):
    n = int(rcvlib.rcv_cv_table_len(beta))
    assert n >= 1
    tab = np.empty(n, np.float32)
    assert rcvlib.rcv_cv_table_fill(beta, tab.ctypes.data, n) == 0
    b = float(np.float32(beta))
    for k in sorted(k for k in {0, 1, 2, 3, n // 2, n - 2, n - 1} if 0 <= k < n):
        # rcv_cv_step: 1.0f - float32(pow((double)beta, k))
        assert tab[k] == np.float32(1.0) - np.float32(b ** k), k
    assert tab[-1] == np.float32(1.0)
    assert n == 1 or tab[-2] != np.float32(1.0)
    # past the table every power gives 1.0f
    assert np.float32(1.0) - np.float32(b ** (n + 50)) == np.float32(1.0)


def test_adam_table_matches_host_arithmetic(rcvlib):
    b1, b2 = 0.9, 0.999
    n = int(rcvlib.rcv_adam_table_len(b1, b2))
    tab = np.empty((n, 2), np.float64)
    assert rcvlib.rcv_adam_table_fill(b1, b2, tab.ctypes.data, n) == 0
    f1, f2 = float(np.float32(b1)), float(np.float32(b2))
    for t in (1, 2, 10, 100, n // 2, n - 1):
        assert tab[t, 0] == math.sqrt(1.0 - f2 ** t)
        assert tab[t, 1] == 1.0 - f1 ** t
    assert tab[-1, 0] == 1.0 and tab[-1, 1] == 1.0
    assert not (tab[-2, 0] == 1.0 and tab[-2, 1] == 1.0)


def test_tables_reject_bad_betas(rcvlib):
    assert rcvlib.rcv_cv_table_len(1.0) == _lib.RCV_ERR_INVALID
    assert rcvlib.rcv_cv_table_len(-0.1) == _lib.RCV_ERR_INVALID
    assert rcvlib.rcv_adam_table_len(0.9, 1.5) == _lib.RCV_ERR_INVALID
    # so close to 1 that the table would exceed 2^22 entries
    assert rcvlib.rcv_cv_table_len(0.99999994) == _lib.RCV_ERR_UNSUPPORTED


def _fake_job(**kw):
    """A structurally valid job description with fake (never dereferenced)
    device pointers, for host-side validation only."""
    j = _lib.BatchJob()
    j.sensor.width, j.sensor.height = 8, 8
    j.dims[:] = [4, 4, 4]
    j.spp = j.spp_grad = 2
    j.max_depth, j.rr_depth = 4, 4
    j.cv_beta1, j.cv_beta2 = 0.9, 0.999
    j.adam_beta1, j.adam_beta2 = 0.9, 0.999
    j.cv_table1 = j.cv_table2 = j.adam_table = 0x1000
    j.cv_table1_len = j.cv_table2_len = j.adam_table_len = 4
    j.density[0], j.density[1] = 0x2000, 0x3000
    j.density_m, j.density_v = 0x4000, 0x5000
    j.target = 0x6000
    for name in ("img", "w_s", "v_n", "mean_x", "mean_y", "var_x", "var_y", "cov"):
        setattr(j.cv, name, 0x7000)
    j.workspace = 0x10000
    for k, v in kw.items():
        if k == "density":
            j.density[0], j.density[1] = v
        elif k == "albedo":
            j.albedo[0], j.albedo[1] = v
        else:
            setattr(j, k, v)
    return j


@pytest.mark.parametrize("change,message", [
    (dict(spp=0), b"spp"),
    (dict(density=(0x2000, 0x2000)), b"density buffers must differ"),
    (dict(albedo=(0x8000, 0)), b"albedo[0] and albedo[1]"),
    (dict(albedo_m=0x9000), b"albedo_m and albedo_v"),
    (dict(albedo_m=0x9000, albedo_v=0xa000), b"moments without an albedo grid"),
    (dict(loss=9), b"loss kind"),
    (dict(workspace=0x10010), b"256-byte aligned"),
    (dict(cv_table1=0), b"CV bias-correction"),
    (dict(cv_beta2=1.0), b"cv betas"),
])
def test_batch_validation_on_host(rcvlib, change, message):
    jobs = (_lib.BatchJob * 2)(_fake_job(), _fake_job(**change))
    ws = rcvlib.rcv_batch_workspace_bytes(jobs, 2)
    h = C.c_void_p()
    rc = rcvlib.rcv_batch_create(jobs, 2, None, 0x100000, ws, C.byref(h), None)
    assert rc == _lib.RCV_ERR_INVALID
    err = rcvlib.rcv_last_error()
    assert message in err and b"job 1" in err, err
    assert not h.value


def test_batch_workspace_bytes(rcvlib):
    a = (_lib.BatchJob * 1)(_fake_job())
    b = (_lib.BatchJob * 2)(_fake_job(), _fake_job(spp=8))
    assert rcvlib.rcv_batch_workspace_bytes(a, 0) == 0
    wa, wb = rcvlib.rcv_batch_workspace_bytes(a, 1), rcvlib.rcv_batch_workspace_bytes(b, 2)
    assert wa > 8 * 8 * 2 * 32 and wb >= wa + 8 * 8 * 8 * 32
    assert rcvlib.rcv_batch_job_workspace_bytes(C.byref(_fake_job())) > 8 * 8 * 12
    assert rcvlib.rcv_batch_kernels_per_step(None) == _lib.RCV_ERR_INVALID


def test_cfg4_mix_is_seeded_and_in_range():
    m1, m2 = batch.cfg4_mix(32), batch.cfg4_mix(32)
    assert m1 == m2 and len(m1) == 32
    assert {m["grid"] for m in m1} <= {16, 32, 64, 128}
    assert {m["res"] for m in m1} <= {64, 128, 256, 512}
    assert {m["spp"] for m in m1} <= {4, 8, 16}
    assert all(m["max_depth"] == 32 for m in m1)


# ------------------------------------------------------------------- GPU
def plain_setup(device, dens, alb, res, depth, lr, spp, adjoint="tape"):
    scene = rcv.load_dict(scenes.scene_dict(dens, alb, res=res, spp=spp), device=device)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath", "max_depth": depth,
                                                         "rr_depth": depth, "adjoint": adjoint}})
    opt = rcv.ad.Adam(lr=lr)
    opt[scenes.DENSITY_KEY] = dens
    opt.set_bounds(scenes.DENSITY_KEY, 0.0, 250.0)
    if not np.isscalar(alb):
        opt[scenes.ALBEDO_KEY] = alb
        opt.set_bounds(scenes.ALBEDO_KEY, 0.0, 1.0)
    params.update(opt)
    params.update(opt)
    return scene, params, integ, opt


def plain_step(scene, params, integ, opt, target, seed, spp):
    params.update(opt)
    img = rcv.render(scene, params, integrator=integ, seed=seed, spp=spp)
    loss = rcv.l2_loss(img, target)
    loss.backward()
    opt.step()
    return float(loss.detach())


JOBS = [  # grid, res, spp, depth, albedo grid
    (16, 32, 4, 8, True),
    (8, 24, 2, 6, False),
    (12, 20, 3, 10, False),
]


def build_pair(cuda, k, lr=0.02):
    D, res, spp, depth, agrid = JOBS[k]
    true = scenes.blob_density(D, 100 + k)
    dens = (0.7 * true).astype(np.float32)
    alb = scenes.albedo_grid(D, 100 + k) if agrid else 0.8
    ref_scene = rcv.load_dict(scenes.scene_dict(true, alb, res=res), device=cuda)
    target = rcv.load_dict({"type": "prbvolpath", "max_depth": depth, "rr_depth": depth}).render(
        ref_scene, 0, seed=999, spp=64)
    alb0 = np.full_like(alb, 0.5) if agrid else alb
    plain = plain_setup(cuda, dens, alb0, res, depth, lr, spp)
    job = batch.CVJob.from_scene(plain[0], plain[1], plain[2], plain[3], target, spp=spp, seed=40 + 7 * k,
                                 keep_images=True)
    return plain, job, target, spp, 40 + 7 * k


def rel_l2(a, b):
    a = a.double().cpu()
    b = b.double().cpu()
    return float(torch.linalg.norm(a - b) / max(torch.linalg.norm(b), 1e-30))


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_matches_plain_api(cuda, use_graph):
    pairs = [build_pair(cuda, k) for k in range(len(JOBS))]
    b = batch.BatchedCV([p[1] for p in pairs], use_graph=use_graph)
    b.step()
    torch.cuda.synchronize()
    for (scene, params, integ, opt), job, target, spp, seed in pairs:
        loss = plain_step(scene, params, integ, opt, target, seed, spp)
        state = integ.cv
        H, F = job.primal_images()
        assert torch.equal(H, state.H) and torch.equal(F, state.F)
        assert torch.equal(job.image(), state.img)
        st = job.status()
        assert st["it"] == 1 and st["welford_count"] == 0 and st["adam_t"] == 1
        assert abs(st["loss"] - loss) <= 1e-6 * abs(loss)
        m_plain = opt.state[scenes.DENSITY_KEY][1].reshape(job.density_m.shape)
        assert rel_l2(job.density_m, m_plain) <= 1e-5
        if job.albedo_m is not None:
            assert rel_l2(job.albedo_m, opt.state[scenes.ALBEDO_KEY][1]) <= 1e-5
        p_plain = opt[scenes.DENSITY_KEY].detach().reshape(job.params().shape)
        close = (job.params() - p_plain).abs() <= 1e-6 * (1.0 + p_plain.abs())
        assert float(close.float().mean()) >= 0.99
    # more steps: both forms evolve; parameters drift apart only where
    # reordered atomics flipped the sign of a near-zero gradient
    b.step(3)
    for (scene, params, integ, opt), job, target, spp, seed in pairs:
        for it in range(1, 4):
            loss = plain_step(scene, params, integ, opt, target, seed + it, spp)
        st = job.status()
        assert st["welford_count"] == 3 and st["adam_t"] == 4
        assert abs(st["loss"] - loss) <= 2e-2 * loss
        assert abs(float(job.image().mean() / integ.cv.img.mean()) - 1.0) <= 5e-3
        assert rel_l2(job.params(), opt[scenes.DENSITY_KEY].detach().reshape(job.params().shape)) <= 1e-2
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [False, True])
def test_single_path_jobs_bitwise_over_many_steps(cuda, use_graph):
    """With one path per step (1x1 film, spp 1) and the replay adjoint every
    gradient atomic of a job comes from one thread in program order, so the
    whole optimisation is deterministic: parameters, moments, weights,
    statistics and images of the batched and the plain form stay
    bit-identical over many steps (this exercises the device-side CV and
    Adam bias-correction tables, and the batched supergrid of the third
    job).  The tape adjoint scatters a path's events from several threads."""
    pairs = []
    for k, (D, agrid, factor) in enumerate([(6, True, 0), (5, False, 0), (12, False, 4)]):
        true = scenes.blob_density(D, 60 + k)
        alb = scenes.albedo_grid(D, 60 + k) if agrid else 0.8
        target = torch.full((1, 1, 3), 0.3 + 0.1 * k, device=cuda)
        alb0 = np.full_like(alb, 0.5) if agrid else alb
        plain = plain_setup(cuda, (0.5 * true).astype(np.float32), alb0, 1, 16, 0.05, 1, adjoint="replay")
        if factor:  # a majorant supergrid on the third job
            plain[0].named_shapes()["object"].interior_medium().set_majorant_resolution_factor(factor)
        job = batch.CVJob.from_scene(*plain, target, spp=1, seed=3 + k, keep_images=True)
        pairs.append((plain, job, target, 3 + k))
    b = batch.BatchedCV([p[1] for p in pairs], batch.LaunchOptions(adjoint="replay"), use_graph=use_graph)
    for it in range(8):
        b.step()
        for (scene, params, integ, opt), job, target, seed in pairs:
            loss = plain_step(scene, params, integ, opt, target, seed + it, 1)
            assert torch.equal(job.image(), integ.cv.img), it
            assert torch.equal(job.cv_state[1], integ.cv.w_s) and torch.equal(job.cv_state[2], integ.cv.v_n)
            p_plain = opt[scenes.DENSITY_KEY].detach().reshape(job.params().shape)
            assert torch.equal(job.params(), p_plain), it
            assert torch.equal(job.density_m, opt.state[scenes.DENSITY_KEY][1].reshape(job.density_m.shape))
            if job.albedo_m is not None:
                assert torch.equal(job.albedo_params(), opt[scenes.ALBEDO_KEY].detach())
            assert abs(job.status()["loss"] - loss) <= 1e-6 * max(abs(loss), 1e-30)
    assert pairs[0][1].status()["welford_count"] == 7
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("per_path", [0, 2])
def test_batch_tape_matches_replay(cuda, per_path):
    """One batched step with the tape adjoint and one with the replay tasks:
    the same images, and first Adam moments (the gradients) within the
    reordering of float atomics; with 2 tape slots per path most paths are
    replayed whole, and the second job has a majorant supergrid (the tape
    then keeps each event's majorant)."""
    pairs = [build_pair(cuda, k) for k in range(len(JOBS))]
    if per_path == 2:  # a majorant supergrid on one job: the tape keeps every event's majorant
        pairs[1][0][0].named_shapes()["object"].interior_medium().set_majorant_resolution_factor(4)
        pairs[1] = (pairs[1][0], batch.CVJob.from_scene(*pairs[1][0], pairs[1][2], spp=pairs[1][3], seed=pairs[1][4],
                                                        keep_images=True), pairs[1][2], pairs[1][3], pairs[1][4])
    jobs_t = [p[1] for p in pairs]
    jobs_r = [j.clone() for j in jobs_t]
    bt = batch.BatchedCV(jobs_t, batch.LaunchOptions(tape_events_per_path=per_path), use_graph=False)
    br = batch.BatchedCV(jobs_r, batch.LaunchOptions(adjoint="replay"), use_graph=False)
    bt.step()
    br.step()
    torch.cuda.synchronize()
    for a, b in zip(jobs_t, jobs_r):
        assert torch.equal(a.image(), b.image())
        assert rel_l2(a.density_m, b.density_m) <= 1e-5
        if a.albedo_m is not None:
            assert rel_l2(a.albedo_m, b.albedo_m) <= 1e-5
    bt.close()
    br.close()


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [False, True])
def test_batch_paired_tracers_match_two_streams(cuda, use_graph):
    """The two-state and tape radiance passes of all jobs in one paired
    launch (the default) or as two launches on two streams: the same images
    bit for bit, gradients (first Adam moments) within the reordering of
    float atomics, over two steps (captured into a graph or not); one
    kernel launch fewer per step when paired."""
    pairs = [build_pair(cuda, k) for k in range(len(JOBS))]
    jobs_p = [p[1] for p in pairs]
    jobs_s = [j.clone() for j in jobs_p]
    bp = batch.BatchedCV(jobs_p, batch.LaunchOptions(), use_graph=use_graph)
    bs = batch.BatchedCV(jobs_s, batch.LaunchOptions(pair_tracers=False), use_graph=use_graph)
    assert bp.kernels_per_step == bs.kernels_per_step - 1
    for step in range(2):
        bp.step()
        bs.step()
        torch.cuda.synchronize()
        for a, b in zip(jobs_p, jobs_s):
            if step == 0:  # later steps start from parameters that differ by the atomics' rounding
                assert torch.equal(a.primal_images()[0], b.primal_images()[0])
                assert torch.equal(a.primal_images()[1], b.primal_images()[1])
                assert torch.equal(a.image(), b.image())
            else:
                assert rel_l2(a.image(), b.image()) <= 1e-3
            tol = 1e-5 if step == 0 else 1e-3
            assert rel_l2(a.density_m, b.density_m) <= tol
            if a.albedo_m is not None:
                assert rel_l2(a.albedo_m, b.albedo_m) <= tol
    bp.close()
    bs.close()


@pytest.mark.gpu
def test_job_alone_and_in_mix_agree(cuda):
    """The same job stepped alone and inside a mix of uneven jobs: first-step
    images bit-identical, later steps within the atomic-reordering tolerance."""
    pairs = [build_pair(cuda, k) for k in range(len(JOBS))]
    alone = pairs[0][1].clone()
    mix = batch.BatchedCV([p[1] for p in pairs], options=batch.LaunchOptions(batch=16, defer=4))
    solo = batch.BatchedCV([alone], options=batch.LaunchOptions(order="row_major"), use_graph=False)
    mix.step()
    solo.step()
    torch.cuda.synchronize()
    assert torch.equal(pairs[0][1].image(), alone.image())
    assert torch.equal(pairs[0][1].primal_images()[0], alone.primal_images()[0])
    mix.step(4)
    solo.step(4)
    assert abs(float(pairs[0][1].image().mean() / alone.image().mean()) - 1.0) <= 5e-3
    assert rel_l2(pairs[0][1].params(), alone.params()) <= 1e-2
    mix.close()
    solo.close()


@pytest.mark.gpu
def test_gradient_variance_matched(cuda):
    """Per-voxel variance of dL/dtheta over 16 seeds in the plain, batched and
    served forms (matched variance: same spp, spp_grad, max_depth and seeds
    in every form).  Same seeds give the same estimates up to float-atomic
    reordering, so the variances agree far inside 5 %.  lr = 0, so Adam's
    first moment after one step is (1 - beta1) * gradient."""
    D, res, spp, depth, n_seeds = 12, 24, 4, 8, 16
    true = scenes.blob_density(D, 5)
    dens = (0.7 * true).astype(np.float32)
    ref_scene = rcv.load_dict(scenes.scene_dict(true, 0.8, res=res), device=cuda)
    target = rcv.load_dict({"type": "prbvolpath", "max_depth": depth, "rr_depth": depth}).render(
        ref_scene, 0, seed=3, spp=64)
    grads_plain, jobs = [], []
    for s in range(n_seeds):
        scene, params, integ, opt = plain_setup(cuda, dens, 0.8, res, depth, 0.0, spp)
        jobs.append(batch.CVJob.from_scene(scene, params, integ, opt, target, spp=spp, seed=1000 + 31 * s))
        plain_step(scene, params, integ, opt, target, 1000 + 31 * s, spp)
        grads_plain.append(opt.state[scenes.DENSITY_KEY][1].reshape(D, D, D) / 0.1)
    served = [j.clone() for j in jobs]
    b = batch.BatchedCV(jobs)
    b.step()
    server = serve.StepServer(8 * 2**30, device=cuda, max_jobs_per_tick=5, pipeline=2)
    for jid in [server.add_job(j) for j in served]:
        server.submit(jid)
    server.drain()
    server.close()
    gp = torch.stack(grads_plain)
    vp = gp.var(dim=0)
    busy = vp > 1e-3 * vp.max()
    for form in (jobs, served):
        assert all(j.it == 1 for j in form)
        g = torch.stack([j.density_m / np.float32(0.1) for j in form])
        v = g.var(dim=0)
        assert float(v.sum()) > 0
        assert abs(float(v.sum() / vp.sum()) - 1.0) < 0.05
        assert float(((v[busy] / vp[busy] - 1).abs() < 0.05).float().mean()) >= 0.99
        # lr = 0: the parameters did not move
        assert all(torch.equal(j.params(), j.density[(j.it + 1) & 1]) for j in form)
    b.close()


@pytest.mark.gpu
def test_autotune_leaves_jobs_untouched(cuda):
    pairs = [build_pair(cuda, k) for k in range(2)]
    jobs = [p[1] for p in pairs]
    before = [j.params().clone() for j in jobs]
    cands = [batch.LaunchOptions(), batch.LaunchOptions(batch=16), batch.LaunchOptions(order="row_major")]
    best = batch.autotune(jobs, candidates=cands, steps=1, use_cache=False)
    assert best in cands
    assert all(j.it == 0 and j.status()["it"] == 0 for j in jobs)
    assert all(torch.equal(a, j.params()) for a, j in zip(before, jobs))
