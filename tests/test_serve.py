"""Gradient-step serving (recursive_control_variates_gb300.serve).

CPU: admission by HBM budget, tick formation (oldest first, one request per
job per tick, path cap), pipelining and latency bookkeeping, with the batch
plan and the CUDA event replaced by host fakes.

GPU: jobs served under Poisson arrivals with continuous batching give the
same results as the same jobs stepped alone.  Single-path jobs (1x1 film,
spp 1: gradient atomics in program order) are compared bit for bit after
every served step; larger jobs bit for bit on their first step (images do not
depend on the other jobs of a tick) and within 1e-2 relative L2 of the
parameters after several steps (float-atomic reordering, see test_batch)."""
import types

import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import batch, scenes, serve


# ------------------------------------------------------------------- CPU
class FakeJob:
    def __init__(self, nbytes, paths=100, device="cpu"):
        self._n = nbytes
        self.width, self.height, self.spp, self.spp_grad = 1, 1, 1, 1
        self._paths = paths
        self.device = torch.device(device)
        self.steps = 0

    def nbytes(self):
        return self._n

    def paths_per_step(self):
        return self._paths


class FakePlan:
    log = []

    def __init__(self, jobs, options=None, use_graph=True):
        self.jobs = jobs
        self.closed = False
        FakePlan.log.append(("create", tuple(id(j) for j in jobs)))

    def step(self):
        for j in self.jobs:
            j.steps += 1

    def close(self):
        self.closed = True


class FakeEvent:
    pending = []

    def __init__(self):
        self.fired = False
        FakeEvent.pending.append(self)

    def record(self, stream=None):
        pass

    def query(self):
        return self.fired


@pytest.fixture
def fake_cuda(monkeypatch):
    FakePlan.log.clear()
    FakeEvent.pending.clear()
    monkeypatch.setattr(serve.B, "BatchedCV", FakePlan)
    monkeypatch.setattr(serve.torch.cuda, "Event", FakeEvent)
    monkeypatch.setattr(serve.torch.cuda, "current_stream", lambda device=None: None)
    monkeypatch.setattr(serve.torch.cuda, "synchronize", lambda device=None: None)
    clock = types.SimpleNamespace(t=0.0)
    return clock


def fire_all():
    for e in FakeEvent.pending:
        e.fired = True


def test_admission_by_budget(fake_cuda):
    s = serve.StepServer(2500, device="cpu", clock=lambda: fake_cuda.t)
    # per-path scratch of a 1 x 1 x spp 1 job: 32 B primal, 144 B gradient
    # (total radiance, records), 332 B of tape
    scratch = s.job_bytes(FakeJob(0))
    assert scratch == 32 + 144 + 332
    replay = serve.StepServer(2500, device="cpu", options=serve.B.LaunchOptions(adjoint="replay"))
    assert replay.job_bytes(FakeJob(0)) == 32 + 144
    a, b, c = (FakeJob(1000 - scratch) for _ in range(3))  # 1000 B each with scratch
    ja, jb, jc = s.add_job(a), s.add_job(b), s.add_job(c)
    assert s.is_resident(ja) and s.is_resident(jb) and not s.is_resident(jc)
    with pytest.raises(ValueError):
        s.add_job(FakeJob(5000))
    s.submit(jc)
    assert not s.pump()  # a waiting job's requests do not run
    s.remove_job(ja)
    assert s.is_resident(jc)
    assert s.pump()
    fire_all()
    done = s.poll()
    assert [r.job_id for r in done] == [jc] and c.steps == 1


def test_ticks_oldest_first_one_request_per_job(fake_cuda):
    s = serve.StepServer(10**9, device="cpu", max_jobs_per_tick=2, pipeline=3, clock=lambda: fake_cuda.t)
    jobs = [FakeJob(10) for _ in range(3)]
    ids = [s.add_job(j) for j in jobs]
    for t, jid in [(0.0, ids[2]), (0.1, ids[2]), (0.2, ids[0]), (0.3, ids[1])]:
        s.submit(jid, arrival=t)
    assert s.pump() and s.pump() and s.pump() is False  # two ticks cover the 4 requests ... almost
    ticks = list(s.inflight)
    assert ticks[0].job_ids == tuple(sorted((ids[2], ids[0])))  # oldest two jobs, one request each
    assert ticks[1].job_ids == tuple(sorted((ids[2], ids[1])))
    fake_cuda.t = 1.5
    fire_all()
    done = s.poll()
    assert len(done) == 4 and all(r.latency is not None for r in done)
    lat = serve.latency_summary(done)
    assert lat["n"] == 4 and abs(lat["max_ms"] - 1500.0) < 1e-6
    assert [j.steps for j in jobs] == [1, 1, 2]


def test_path_cap_and_plan_reuse(fake_cuda):
    s = serve.StepServer(10**9, device="cpu", max_paths_per_tick=250, pipeline=1, clock=lambda: fake_cuda.t)
    ids = [s.add_job(FakeJob(10, paths=100)) for _ in range(3)]
    for jid in ids:
        s.submit(jid, arrival=0.0)
    assert s.pump() and len(s.inflight[0].job_ids) == 2
    assert not s.pump()  # pipeline depth 1
    fire_all()
    s.poll()
    assert s.pump() and s.inflight[0].job_ids == (ids[2],)
    fire_all()
    s.poll()
    for jid in ids[:2]:
        s.submit(jid)
    s.pump()
    fire_all()
    s.poll()
    for jid in ids[:2]:
        s.submit(jid)
    s.pump()
    assert s.stats.plan_reuses == 1


def test_poisson_arrivals_seeded():
    a = serve.poisson_arrivals(2000.0, 500, range(10), seed=3)
    assert a == serve.poisson_arrivals(2000.0, 500, range(10), seed=3)
    t = np.array([x[0] for x in a])
    assert np.all(np.diff(t) > 0)
    assert 0.2 < t[-1] < 0.3  # 500 arrivals at 2000/s
    assert {x[1] for x in a} <= set(range(10))


# ------------------------------------------------------------------- GPU
def make_job(device, D, res, spp, seed, single_path=False):
    true = scenes.blob_density(D, seed)
    if single_path:
        target = torch.full((1, 1, 3), 0.35, device=device)
        scene = rcv.load_dict(scenes.scene_dict(true, 0.8, res=1), device=device)
    else:
        scene = rcv.load_dict(scenes.scene_dict(true, 0.8, res=res), device=device)
        target = rcv.load_dict({"type": "prbvolpath", "max_depth": 8, "rr_depth": 8}).render(scene, 0, seed=7, spp=32)
    return batch.CVJob(0.6 * true, 0.8, target, scene.sensors()[0], spp=spp, max_depth=8, rr_depth=8, seed=seed * 13,
                       lr=0.03, density_bounds=(0.0, 250.0), device=device)


@pytest.mark.gpu
def test_served_results_same_as_alone(cuda):
    specs = [(6, 1, 1, 1, True), (5, 1, 1, 2, True), (12, 24, 4, 3, False), (16, 32, 2, 4, False)]
    served = [make_job(cuda, D, r, spp, sd, sp) for D, r, spp, sd, sp in specs]
    alone = [j.clone() for j in served]
    server = serve.StepServer(8 * 2**30, device=cuda, max_jobs_per_tick=3, pipeline=2)
    ids = [server.add_job(j) for j in served]
    rng = np.random.default_rng(0)
    steps = 4
    arrivals = [(float(t), ids[k]) for k in range(len(ids)) for t in rng.uniform(0, 0.01, size=steps)]
    reqs = server.run_arrivals(arrivals)
    server.close()
    assert all(r.done is not None for r in reqs) and len(reqs) == steps * len(ids)
    assert server.stats.ticks >= steps and max(server.stats.jobs_per_tick) > 1
    for j, a in zip(served, alone):
        b = batch.BatchedCV([a], use_graph=False)
        b.step(steps)
        b.close()
        assert j.it == a.it == steps
        if j.width == 1:
            assert torch.equal(j.params(), a.params()) and torch.equal(j.image(), a.image())
            assert torch.equal(j.cv_state, a.cv_state)
        else:
            rel = torch.linalg.norm((j.params() - a.params()).double()) / torch.linalg.norm(a.params().double())
            assert float(rel) <= 1e-2
    lat = serve.latency_summary(reqs)
    assert lat["n"] == len(reqs) and lat["p99_ms"] >= lat["p50_ms"] > 0


@pytest.mark.gpu
def test_first_served_step_bitwise(cuda):
    a = make_job(cuda, 12, 24, 4, 9)
    b = make_job(cuda, 16, 20, 2, 10)
    a_alone = a.clone()
    server = serve.StepServer(8 * 2**30, device=cuda)
    ia, ib = server.add_job(a), server.add_job(b)
    server.submit(ia)
    server.submit(ib)
    server.drain()
    server.close()
    solo = batch.BatchedCV([a_alone], use_graph=False)
    solo.step()
    solo.close()
    assert torch.equal(a.image(), a_alone.image())
    assert torch.equal(a.cv_state, a_alone.cv_state)
