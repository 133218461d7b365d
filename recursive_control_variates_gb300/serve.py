"""Gradient-step serving: continuous batching of step requests from many
resident inverse-rendering jobs on one GPU.

Each registered job (``batch.CVJob``) keeps its grids, parameter double
buffer, Adam moments, previous-iterate image and EMA-Welford statistics on the
device for its whole life.  Jobs are admitted by an HBM budget: a job becomes
resident only while the bytes of all resident jobs plus the tracer scratch a
tick of all of them would need fit in the budget; the others wait and are
admitted, in registration order, as resident jobs are removed.

A request asks for one cv_ps step of one job.  The server forms *ticks*: the
pending requests, oldest first, at most one per job, up to
``max_jobs_per_tick`` jobs and ``max_paths_per_tick`` paths.  A tick is one
``BatchedCV`` step over its jobs (one persistent tracer launch per pass for
all of them), so the work of every request admitted to a tick overlaps on the
device.  Requests that arrive while a tick runs join the next one; with
``pipeline`` > 1 the next tick is enqueued behind the running one (stream
order keeps each job's steps sequential) so the host prepares it while the
GPU works.  A request completes when its tick's CUDA event completes;
latency = completion time - arrival time.

A job's result does not depend on which other jobs share its ticks: per job,
a tick performs exactly the single-job step (see ``batch``).
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import batch as B


@dataclass
class Request:
    job_id: int
    arrival: float                 # seconds (server clock)
    done: float | None = None      # completion time (server clock)
    tick: int = -1

    @property
    def latency(self) -> float | None:
        return None if self.done is None else self.done - self.arrival


@dataclass
class _Tick:
    index: int
    job_ids: tuple
    requests: list
    event: torch.cuda.Event
    plan: B.BatchedCV | None
    paths: int
    enqueued: float


@dataclass
class ServerStats:
    completed: int = 0
    paths: int = 0
    ticks: int = 0
    jobs_per_tick: list = field(default_factory=list)
    plan_reuses: int = 0


class StepServer:
    def __init__(self, hbm_budget_bytes: int, device="cuda", max_jobs_per_tick: int = 256,
                 max_paths_per_tick: int | None = None, options: B.LaunchOptions | None = None,
                 use_graph: bool = True, pipeline: int = 2, clock=time.perf_counter):
        self.device = torch.device(device)
        self.budget = int(hbm_budget_bytes)
        self.max_jobs = int(max_jobs_per_tick)
        self.max_paths = int(max_paths_per_tick) if max_paths_per_tick else None
        self.options = options or B.LaunchOptions()
        self.use_graph = bool(use_graph)
        self.pipeline = max(1, int(pipeline))
        self.clock = clock
        self.t0 = clock()
        self.jobs: dict[int, B.CVJob] = {}          # resident
        self.waiting: collections.OrderedDict[int, B.CVJob] = collections.OrderedDict()
        self.pending: dict[int, collections.deque] = {}
        self.inflight: collections.deque[_Tick] = collections.deque()
        self.stats = ServerStats()
        self._next_id = 0
        self._tick = 0
        self._last_plan: B.BatchedCV | None = None
        self._last_ids: tuple = ()

    # ------------------------------------------------------------ memory
    def job_bytes(self, job: B.CVJob) -> int:
        """Resident bytes of a job plus the per-path scratch it adds to a tick:
        32 bytes per primal path (radiance slots), 16 + 2 x 64 bytes per
        gradient path (total radiance, scatter checkpoints or event records
        and their weights), and with the tape adjoint 16 x 20 + 8 + 4 bytes
        more (event slots with their extinction terms, camera-segment weight,
        lost-path list)."""
        npix = job.width * job.height
        per_grad = 144 + (332 if self.options.adjoint == "tape" else 0)
        return job.nbytes() + 32 * npix * job.spp + per_grad * npix * job.spp_grad

    def resident_bytes(self) -> int:
        return sum(self.job_bytes(j) for j in self.jobs.values())

    def _admit_waiting(self) -> None:
        while self.waiting:
            jid, job = next(iter(self.waiting.items()))
            if self.resident_bytes() + self.job_bytes(job) > self.budget:
                break
            self.waiting.popitem(last=False)
            self.jobs[jid] = job

    # -------------------------------------------------------------- jobs
    def add_job(self, job: B.CVJob) -> int:
        """Registers a job; it is resident at once if the budget allows,
        otherwise it waits (its requests queue until it is admitted)."""
        if job.device != self.device:
            raise ValueError("the job lives on another device")
        if self.job_bytes(job) > self.budget:
            raise ValueError(f"job needs {self.job_bytes(job)} bytes, more than the whole budget {self.budget}")
        jid = self._next_id
        self._next_id += 1
        self.pending[jid] = collections.deque()
        self.waiting[jid] = job
        self._admit_waiting()
        return jid

    def remove_job(self, jid: int) -> B.CVJob:
        """Drops a job once its requests are served; frees its budget."""
        if self.pending.get(jid):
            raise RuntimeError(f"job {jid} still has pending requests")
        if any(jid in t.job_ids for t in self.inflight):
            raise RuntimeError(f"job {jid} has a step in flight")
        job = self.jobs.pop(jid, None) or self.waiting.pop(jid)
        del self.pending[jid]
        if jid in self._last_ids:
            self._drop_plan()
        self._admit_waiting()
        return job

    def is_resident(self, jid: int) -> bool:
        return jid in self.jobs

    # ----------------------------------------------------------- requests
    def now(self) -> float:
        return self.clock() - self.t0

    def submit(self, jid: int, arrival: float | None = None) -> Request:
        if jid not in self.pending:
            raise KeyError(f"unknown job {jid}")
        r = Request(jid, self.now() if arrival is None else float(arrival))
        self.pending[jid].append(r)
        return r

    def _form_tick(self):
        cands = [(q[0].arrival, jid) for jid, q in self.pending.items() if q and jid in self.jobs]
        cands.sort()
        chosen, paths = [], 0
        for _, jid in cands:
            if len(chosen) >= self.max_jobs:
                break
            p = self.jobs[jid].paths_per_step()
            if chosen and self.max_paths is not None and paths + p > self.max_paths:
                continue
            chosen.append(jid)
            paths += p
        return tuple(sorted(chosen)), paths

    def _drop_plan(self):
        if self._last_plan is not None and not any(t.plan is self._last_plan for t in self.inflight):
            self._last_plan.close()
        self._last_plan, self._last_ids = None, ()

    def pump(self) -> bool:
        """Enqueues the next tick if the pipeline has room and requests wait."""
        if len(self.inflight) >= self.pipeline:
            return False
        ids, paths = self._form_tick()
        if not ids:
            return False
        if ids == self._last_ids and self._last_plan is not None:
            plan = self._last_plan
            self.stats.plan_reuses += 1
            # a plan that is stepped again is worth capturing as a CUDA graph
            plan.use_graph = self.use_graph
        else:
            old = self._last_plan
            # most ticks form a new plan that runs once: its launches are
            # enqueued directly, without the cost of capturing a graph
            plan = B.BatchedCV([self.jobs[j] for j in ids], options=self.options, use_graph=False)
            self._last_plan, self._last_ids = plan, ids
            if old is not None and not any(t.plan is old for t in self.inflight):
                old.close()
        reqs = [self.pending[j].popleft() for j in ids]
        plan.step()
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.device))
        for r in reqs:
            r.tick = self._tick
        self.inflight.append(_Tick(self._tick, ids, reqs, ev, plan, paths, self.now()))
        self._tick += 1
        self.stats.ticks += 1
        self.stats.jobs_per_tick.append(len(ids))
        return True

    def poll(self) -> list:
        """Completes the in-flight ticks whose event has fired (in order)."""
        done = []
        while self.inflight and self.inflight[0].event.query():
            t = self.inflight.popleft()
            now = self.now()
            for r in t.requests:
                r.done = now
            self.stats.completed += len(t.requests)
            self.stats.paths += t.paths
            done.extend(t.requests)
            if t.plan is not self._last_plan and not any(x.plan is t.plan for x in self.inflight):
                t.plan.close()
        return done

    def busy(self) -> bool:
        return bool(self.inflight) or any(q for jid, q in self.pending.items() if jid in self.jobs)

    def drain(self, idle_sleep: float = 5e-5) -> None:
        while self.busy():
            self.pump()
            if not self.poll():
                time.sleep(idle_sleep)

    # ---------------------------------------------------------- workloads
    def run_arrivals(self, arrivals, idle_sleep: float = 5e-5) -> list:
        """Open-loop replay of (time, job_id) arrivals on the server clock
        (times relative to the call); returns the requests once all are
        served."""
        arrivals = sorted(arrivals)
        start = self.now()
        reqs, k = [], 0
        while k < len(arrivals) or self.busy():
            now = self.now() - start
            while k < len(arrivals) and arrivals[k][0] <= now:
                t, jid = arrivals[k]
                reqs.append(self.submit(jid, arrival=start + t))
                k += 1
            progressed = self.pump()
            progressed = bool(self.poll()) or progressed
            if not progressed:
                time.sleep(idle_sleep)
        return reqs

    def close(self) -> None:
        torch.cuda.synchronize(self.device)
        while self.inflight:
            self.poll()
        self._drop_plan()


def poisson_arrivals(rate_hz: float, n: int, job_ids, seed: int = 0):
    """n arrivals of a Poisson process of the given rate, each for a job drawn
    uniformly from job_ids."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate_hz, size=n))
    ids = rng.choice(np.asarray(list(job_ids)), size=n)
    return [(float(a), int(b)) for a, b in zip(t, ids)]


def latency_summary(reqs) -> dict:
    lat = np.array([r.latency for r in reqs if r.latency is not None], np.float64) * 1e3
    if lat.size == 0:
        return {"p50_ms": None, "p99_ms": None, "mean_ms": None, "n": 0}
    return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "max_ms": float(lat.max()), "n": int(lat.size)}


def cfg5_mix(n_small: int = 64, n_large: int = 8, seed: int = 5):
    """The served configuration's jobs: n_small from the batched size mix plus
    n_large at 256^3 density, 1024^2 film, spp 16 (depth 32)."""
    small = B.cfg4_mix(n_small, seed=seed)
    large = [dict(grid=256, res=1024, spp=16, max_depth=32) for _ in range(n_large)]
    return small + large
