"""Batched cv_ps optimisation: many independent inverse-rendering jobs of
uneven grid, film and sample counts advanced together (librcv ``rcv_batch_*``).

One batch step is one step of every job, in six kernel launches whatever the
number of jobs (prologue, medium packing, ONE persistent two-state tracer
launch over all jobs' paths, reduce + control variate + loss, ONE persistent
adjoint launch, gradient fold + Adam + clamp).  All per-step values are
derived on the device from per-job counters, so the step is captured once
into a CUDA graph and replayed.  Per job, a step is the loop body of the
reference's cv_ps optimisation (optimize.py:105-131: params.update, mi.render
with the ``cv`` integrator around ``twostateprbvolpath``, loss, dr.backward,
Adam + clamp) with seed = seed_base + it and the default gradient seed.

``CVJob`` owns one job's device state (parameters, Adam moments, control
variate images and statistics, target, workspace); ``BatchedCV`` plans and
steps a list of jobs; ``autotune`` picks the tracer launch options (paths per
queue fetch, resident blocks per SM, deferral threshold, pixel order) for a
size mix by timing steps on copies of the jobs.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .utils import stream_handle

_INF = float("inf")


def _aligned(buf: torch.Tensor) -> int:
    return (buf.data_ptr() + 255) & ~255


# --------------------------------------------------------- bias-correction tables
_TABLES: dict = {}


def cv_table(beta: float, device) -> torch.Tensor:
    """Device table d[k] = 1 - float32(beta^k) (rcv_cv_table_fill), cached."""
    key = ("cv", float(np.float32(beta)), torch.device(device))
    t = _TABLES.get(key)
    if t is None:
        lib = _lib.load()
        n = int(lib.rcv_cv_table_len(float(beta)))
        if n < 0:
            _lib.check(n, "rcv_cv_table_len")
        host = np.empty(n, np.float32)
        _lib.check(lib.rcv_cv_table_fill(float(beta), host.ctypes.data, n), "rcv_cv_table_fill")
        t = torch.from_numpy(host).to(device)
        _TABLES[key] = t
    return t


def adam_table(beta1: float, beta2: float, device) -> torch.Tensor:
    """Device table of (sqrt(1 - beta2^t), 1 - beta1^t) (rcv_adam_table_fill), cached."""
    key = ("adam", float(np.float32(beta1)), float(np.float32(beta2)), torch.device(device))
    t = _TABLES.get(key)
    if t is None:
        lib = _lib.load()
        n = int(lib.rcv_adam_table_len(float(beta1), float(beta2)))
        if n < 0:
            _lib.check(n, "rcv_adam_table_len")
        host = np.empty((n, 2), np.float64)
        _lib.check(lib.rcv_adam_table_fill(float(beta1), float(beta2), host.ctypes.data, n), "rcv_adam_table_fill")
        t = torch.from_numpy(host).to(device)
        _TABLES[key] = t
    return t


# ------------------------------------------------------------------------ jobs
class CVJob:
    """One cv_ps optimisation job resident on the device.

    density: (Dz, Dy, Dx[, 1]) initial grid; albedo: a float, an RGB triple or
    a (Dz, Dy, Dx, 3) grid; target: (H, W, 3) image; sensor: a
    ``PerspectiveSensor`` (or anything with ``c_struct()``) whose film gives
    H, W.  The remaining keywords mirror the plain API: the nested integrator's
    ``max_depth`` / ``rr_depth`` / ``hide_emitters``, the ``cv`` plugin's
    ``warmup`` / ``beta1`` / ``beta2`` (and ``meta``'s ``pre_update``), the
    optimiser's ``lr`` / betas / epsilon and clamp ranges, and the loss.
    ``optimize_albedo`` (default: when the albedo is a grid) adds the albedo
    grid to the optimised variables; ``majorant_factor`` > 0 gives the medium
    a majorant supergrid (the reference's ``majorant_resolution_factor``);
    ``box`` (a ``core.BoxTransform``, default the unit cube) places the grid
    in the world.  The sensor may be a ``batch`` sensor."""

    def __init__(self, density, albedo, target, sensor, *, spp: int, spp_grad: int = 0, max_depth: int = 6,
                 rr_depth: int = 5, hide_emitters: bool = False, scale: float = 1.0, seed: int = 0,
                 lr: float = 0.02, adam_betas=(0.9, 0.999), adam_eps: float = 1e-8,
                 density_bounds=(-_INF, _INF), albedo_bounds=(-_INF, _INF), warmup: int = 1, beta1: float = 0.9,
                 beta2: float = 0.999, pre_update: bool = False, loss: str = "l2", optimize_albedo=None,
                 keep_images: bool = False, majorant_factor: int = 0, box=None, device="cuda"):
        lib = _lib.load()
        self.device = torch.device(device)
        dev = self.device
        d = torch.as_tensor(np.asarray(density, np.float32) if not isinstance(density, torch.Tensor) else density)
        d = d.detach().to(dev, torch.float32)
        if d.dim() == 4:
            if d.shape[-1] != 1:
                raise ValueError("density must have shape (Dz, Dy, Dx) or (Dz, Dy, Dx, 1)")
            d = d[..., 0]
        if d.dim() != 3:
            raise ValueError("density must have shape (Dz, Dy, Dx) or (Dz, Dy, Dx, 1)")
        self.dims = (int(d.shape[2]), int(d.shape[1]), int(d.shape[0]))  # Dx, Dy, Dz
        self.density = torch.stack([d, d]).contiguous()  # double buffer, both = initial state
        self.density_m = torch.zeros_like(d)
        self.density_v = torch.zeros_like(d)
        alb = albedo if isinstance(albedo, torch.Tensor) else np.asarray(albedo, np.float32)
        self.albedo = None
        self.albedo_value = (0.0, 0.0, 0.0)
        if alb.ndim >= 3:
            a = torch.as_tensor(alb).detach().to(dev, torch.float32)
            if tuple(a.shape) != (self.dims[2], self.dims[1], self.dims[0], 3):
                raise ValueError(f"albedo grid must have shape (Dz, Dy, Dx, 3), got {tuple(a.shape)}")
            self.albedo = torch.stack([a, a]).contiguous()
        else:
            v = np.broadcast_to(np.asarray(alb, np.float32), (3,))
            self.albedo_value = tuple(float(x) for x in v)
        if optimize_albedo is None:
            optimize_albedo = self.albedo is not None
        if optimize_albedo and self.albedo is None:
            raise ValueError("optimize_albedo needs an albedo grid")
        self.albedo_m = torch.zeros_like(self.albedo[0]) if optimize_albedo else None
        self.albedo_v = torch.zeros_like(self.albedo[0]) if optimize_albedo else None
        self.sensor = sensor
        s = sensor.c_struct()
        self.width, self.height = int(s.width), int(s.height)
        tgt = torch.as_tensor(target).detach().to(dev, torch.float32).contiguous()
        if tuple(tgt.shape) != (self.height, self.width, 3):
            raise ValueError(f"target has shape {tuple(tgt.shape)}, expected {(self.height, self.width, 3)}")
        self.target = tgt
        self.cv_state = torch.zeros((8, self.height, self.width, 3), dtype=torch.float32, device=dev)
        self.images = (torch.zeros((2, self.height, self.width, 3), dtype=torch.float32, device=dev)
                       if keep_images else None)
        self.spp = int(spp)
        self.spp_grad = int(spp_grad) if spp_grad else int(spp)
        if loss not in ("l2", "l1"):
            raise ValueError(f"unknown loss {loss!r}")
        self.loss_kind = loss
        self.seed = int(seed)
        self._tables = (cv_table(beta1, dev), cv_table(beta2, dev), adam_table(adam_betas[0], adam_betas[1], dev))

        j = _lib.BatchJob()
        j.sensor = s
        j.dims[:] = list(self.dims)
        j.scale = float(scale)
        j.albedo_value[:] = list(self.albedo_value)
        j.spp, j.spp_grad = self.spp, self.spp_grad
        j.max_depth, j.rr_depth, j.hide_emitters = int(max_depth), int(rr_depth), int(bool(hide_emitters))
        j.seed_base = self.seed & 0xFFFFFFFF
        j.warmup, j.pre_update = int(warmup), int(bool(pre_update))
        j.cv_beta1, j.cv_beta2 = float(beta1), float(beta2)
        j.cv_table1, j.cv_table2 = self._tables[0].data_ptr(), self._tables[1].data_ptr()
        j.cv_table1_len, j.cv_table2_len = self._tables[0].numel(), self._tables[1].numel()
        j.loss = _lib.LOSS_L2 if loss == "l2" else _lib.LOSS_L1
        j.lr, j.adam_beta1, j.adam_beta2, j.adam_eps = float(lr), float(adam_betas[0]), float(adam_betas[1]), float(
            adam_eps)
        j.density_lo, j.density_hi = float(density_bounds[0]), float(density_bounds[1])
        j.albedo_lo, j.albedo_hi = float(albedo_bounds[0]), float(albedo_bounds[1])
        j.adam_table, j.adam_table_len = self._tables[2].data_ptr(), self._tables[2].shape[0]
        if int(majorant_factor) < 0:
            raise ValueError("majorant_factor must be >= 0")
        j.majorant_factor = int(majorant_factor)
        if box is not None:  # a core.BoxTransform: the medium's to_world
            j.box_min[:] = [float(np.float32(v)) for v in box.box_min]
            j.box_size[:] = [float(np.float32(v)) for v in box.box_size]
        j.density[0], j.density[1] = self.density[0].data_ptr(), self.density[1].data_ptr()
        if self.albedo is not None:
            j.albedo[0], j.albedo[1] = self.albedo[0].data_ptr(), self.albedo[1].data_ptr()
        j.density_m, j.density_v = self.density_m.data_ptr(), self.density_v.data_ptr()
        if self.albedo_m is not None:
            j.albedo_m, j.albedo_v = self.albedo_m.data_ptr(), self.albedo_v.data_ptr()
        j.target = self.target.data_ptr()
        for k, name in enumerate(("img", "w_s", "v_n", "mean_x", "mean_y", "var_x", "var_y", "cov")):
            setattr(j.cv, name, self.cv_state[k].data_ptr())
        if self.images is not None:
            j.img_old, j.img_new = self.images[0].data_ptr(), self.images[1].data_ptr()
        nbytes = int(lib.rcv_batch_job_workspace_bytes(C.byref(j)))
        if nbytes <= 0:
            raise ValueError("invalid job description")
        self.workspace = torch.empty(nbytes + 256, dtype=torch.uint8, device=dev)
        j.workspace = _aligned(self.workspace)
        self.c = j
        self._status_offset = j.workspace - self.workspace.data_ptr()
        self.it = 0  # host mirror of the device step counter
        _lib.check(lib.rcv_batch_job_init(C.byref(j), stream_handle(dev)), "rcv_batch_job_init")

    # ------------------------------------------------------------ from plain API
    @classmethod
    def from_scene(cls, scene, params, integrator, opt, target, *, spp: int, spp_grad: int = 0, seed: int = 0,
                   loss: str = "l2", keep_images: bool = False):
        """Job of a scene set up for the plain API: ``scene`` with a
        ``twostatemedium`` (load_dict), its ``params`` (traverse), a ``cv`` /
        ``meta`` integrator (load_dict) and an ``ad.Adam`` holding the
        medium's density (and optionally albedo) variables."""
        from .core import TwoStateMedium

        if getattr(integrator, "method", "cv_ps") != "cv_ps":
            raise ValueError("the batched engine runs the cv_ps method")
        inner = integrator.integrator
        medium = inner.medium_of(scene)
        if not isinstance(medium, TwoStateMedium):
            raise RuntimeError("No TwoStateMedium found in the scene!")
        if hasattr(scene, "envmap") and scene.envmap() is not None:
            raise ValueError("the batched engine renders under the constant environment only (the scene has an envmap)")
        keys = {}
        for key in opt.keys():
            owner, sub = params.owner_of(key)
            if owner is medium:
                keys[sub] = key
        if "sigma_t.data" not in keys:
            raise ValueError("the optimiser must hold the medium's density (sigma_t.data)")
        dkey = keys["sigma_t.data"]
        new = medium.new
        if new.has_albedo_grid:
            akey = keys.get("albedo.data")
            albedo = opt[akey].detach() if akey else new.albedo_grid
        else:
            albedo, akey = new.albedo_value, None
        lr_of = lambda k: opt.lr_per_key.get(k, opt.lr)  # noqa: E731
        if akey is not None and lr_of(akey) != lr_of(dkey):
            raise ValueError("the batched engine uses one learning rate per job")
        return cls(
            opt[dkey].detach(), albedo, target, scene.sensors()[0], spp=spp, spp_grad=spp_grad,
            max_depth=inner.max_depth, rr_depth=inner.rr_depth, hide_emitters=inner.hide_emitters, scale=new.scale,
            seed=seed, lr=lr_of(dkey), adam_betas=(opt.beta_1, opt.beta_2), adam_eps=opt.epsilon,
            density_bounds=opt.bounds.get(dkey, (-_INF, _INF)),
            albedo_bounds=opt.bounds.get(akey, (-_INF, _INF)) if akey else (-_INF, _INF),
            warmup=integrator.warmup, beta1=integrator.beta1, beta2=integrator.beta2,
            pre_update=getattr(integrator, "pre_update", False), loss=loss, optimize_albedo=akey is not None,
            keep_images=keep_images, majorant_factor=medium.majorant_resolution_factor(), box=new.box,
            device=medium.device,
        )

    # ---------------------------------------------------------------- state
    def params(self) -> torch.Tensor:
        """Current density theta_it, (Dz, Dy, Dx) view of the double buffer."""
        return self.density[self.it & 1]

    def albedo_params(self) -> torch.Tensor | None:
        return None if self.albedo is None else self.albedo[self.it & 1]

    def image(self) -> torch.Tensor:
        """Control-variate image G of the last step (H, W, 3)."""
        return self.cv_state[0]

    def primal_images(self):
        """(H, F) of the last step when the job keeps them."""
        if self.images is None:
            raise RuntimeError("the job was created with keep_images=False")
        return self.images[0], self.images[1]

    def status(self) -> dict:
        """Device status (synchronises the stream): it, welford_count, adam_t, loss."""
        raw = self.workspace[self._status_offset:self._status_offset + C.sizeof(_lib.BatchJobStatus)].cpu().numpy()
        st = _lib.BatchJobStatus.from_buffer_copy(raw.tobytes())
        return {"it": st.it, "welford_count": st.welford_count, "adam_t": st.adam_t, "loss": st.loss,
                "loss_sum": st.loss_sum}

    def paths_per_step(self) -> int:
        return self.width * self.height * (self.spp + self.spp_grad)

    def nbytes(self) -> int:
        """Device bytes this job holds (grids, moments, images, statistics, workspace)."""
        ts = [self.density, self.density_m, self.density_v, self.target, self.cv_state, self.workspace, self.albedo,
              self.albedo_m, self.albedo_v, self.images]
        return int(sum(t.numel() * t.element_size() for t in ts if t is not None))

    def clone(self) -> "CVJob":
        """Independent copy of the job's device state (same step count)."""
        other = CVJob.__new__(CVJob)
        other.__dict__.update(self.__dict__)
        for name in ("density", "density_m", "density_v", "albedo", "albedo_m", "albedo_v", "target", "cv_state",
                     "images"):
            t = getattr(self, name)
            setattr(other, name, None if t is None else t.clone())
        other.workspace = torch.empty_like(self.workspace)
        j = _lib.BatchJob.from_buffer_copy(bytes(self.c))
        j.density[0], j.density[1] = other.density[0].data_ptr(), other.density[1].data_ptr()
        if other.albedo is not None:
            j.albedo[0], j.albedo[1] = other.albedo[0].data_ptr(), other.albedo[1].data_ptr()
        j.density_m, j.density_v = other.density_m.data_ptr(), other.density_v.data_ptr()
        if other.albedo_m is not None:
            j.albedo_m, j.albedo_v = other.albedo_m.data_ptr(), other.albedo_v.data_ptr()
        j.target = other.target.data_ptr()
        for k, name in enumerate(("img", "w_s", "v_n", "mean_x", "mean_y", "var_x", "var_y", "cov")):
            setattr(j.cv, name, other.cv_state[k].data_ptr())
        if other.images is not None:
            j.img_old, j.img_new = other.images[0].data_ptr(), other.images[1].data_ptr()
        j.workspace = _aligned(other.workspace)
        other.c = j
        other._status_offset = j.workspace - other.workspace.data_ptr()
        # same aligned offset in both workspaces: copy the header, order, ...
        n = self.workspace.numel() - max(self._status_offset, other._status_offset)
        other.workspace[other._status_offset:other._status_offset + n].copy_(
            self.workspace[self._status_offset:self._status_offset + n])
        # the pixel order is part of the copied workspace; the medium cells
        # are rebuilt by every step
        return other


# ---------------------------------------------------------------------- batch
@dataclass(frozen=True)
class LaunchOptions:
    """Tracer launch options of a batch (results do not depend on them)."""

    batch: int = 64          # paths a warp claims per queue fetch
    blocks_per_sm: int = 0   # resident tracer blocks per SM (0 = occupancy limit)
    defer: int = 8           # lanes that must wait before a deferred branch runs
    order: str = "cost"      # pixel hand-out order: cost | longest_first | row_major
    count_events: bool = False  # accumulate the tracer event counts (counters())
    adjoint: str = "tape"    # gradient from the event tape | replayed segments ("replay")
    tape_events_per_path: int = 0  # tape slots per path, 0 = 16 (testing: fewer, paths are replayed)
    pair_tracers: bool = True  # two-state and adjoint radiance passes in one launch (else two streams)

    def c_struct(self) -> _lib.VolpathOptions:
        o = _lib.VolpathOptions()
        o.batch, o.blocks_per_sm, o.defer = self.batch, self.blocks_per_sm, self.defer
        o.count_events = int(self.count_events)
        if self.order not in _lib.ORDERS:
            raise ValueError(f"unknown pixel order {self.order!r}")
        o.order = _lib.ORDERS[self.order]
        if self.adjoint not in _lib.ADJOINTS:
            raise ValueError(f"unknown adjoint {self.adjoint!r}")
        o.adjoint = _lib.ADJOINTS[self.adjoint]
        o.tape_events_per_path = self.tape_events_per_path
        o.separate_tracers = 0 if self.pair_tracers else 1
        return o


class BatchedCV:
    """Plan of a fixed list of jobs; ``step()`` advances every job by one
    cv_ps step (through a CUDA graph when ``use_graph``)."""

    def __init__(self, jobs, options: LaunchOptions | None = None, use_graph: bool = True):
        if not jobs:
            raise ValueError("a batch needs at least one job")
        self.jobs = list(jobs)
        self.device = self.jobs[0].device
        if any(j.device != self.device for j in self.jobs):
            raise ValueError("all jobs of a batch must live on one device")
        if len({id(j) for j in self.jobs}) != len(self.jobs):
            raise ValueError("a job may appear only once in a batch")
        self.options = options or LaunchOptions()
        self.use_graph = bool(use_graph)
        lib = _lib.load()
        n = len(self.jobs)
        self._arr = (_lib.BatchJob * n)(*[j.c for j in self.jobs])
        need = int(lib.rcv_batch_workspace_bytes(self._arr, n))
        if need <= 0:
            raise ValueError("invalid batch")
        self.workspace = torch.empty(need + 256, dtype=torch.uint8, device=self.device)
        self._handle = C.c_void_p()
        o = self.options.c_struct()
        _lib.check(lib.rcv_batch_create(self._arr, n, C.byref(o), _aligned(self.workspace), need,
                                        C.byref(self._handle), stream_handle(self.device)), "rcv_batch_create")
        ptr = int(lib.rcv_batch_counters(self._handle))
        off = ptr - self.workspace.data_ptr()
        self._counters = self.workspace[off:off + 16 * 8].view(torch.int64).view(2, _lib.COUNTER_COUNT)
        self.kernels_per_step = int(lib.rcv_batch_kernels_per_step(self._handle))

    def step(self, steps: int = 1) -> None:
        if self._handle is None:
            raise RuntimeError("the batch was closed")
        lib = _lib.load()
        st = stream_handle(self.device)
        for _ in range(int(steps)):
            _lib.check(lib.rcv_batch_step(self._handle, int(self.use_graph), st), "rcv_batch_step")
            for j in self.jobs:
                j.it += 1

    def counters(self) -> torch.Tensor:
        """(2, RCV_COUNTER_COUNT) int64 device counters: two-state, adjoint."""
        return self._counters

    def paths_per_step(self) -> int:
        return sum(j.paths_per_step() for j in self.jobs)

    def close(self) -> None:
        if self._handle is not None:
            _lib.load().rcv_batch_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------- autotune
_TUNED: dict = {}


def mix_signature(jobs) -> tuple:
    """Key of a size mix: sorted (grid, film, spp, spp_grad, depth) of the jobs."""
    return tuple(sorted((j.dims, j.width, j.height, j.spp, j.spp_grad, j.c.max_depth, j.albedo is not None)
                        for j in jobs))


def default_candidates():
    """One-knob-at-a-time sweep around the defaults."""
    base = LaunchOptions()
    out = [base]
    for b in (16, 32, 128, 256):
        out.append(LaunchOptions(batch=b))
    for d in (2, 4, 16):
        out.append(LaunchOptions(defer=d))
    for k in (2, 3, 4):
        out.append(LaunchOptions(blocks_per_sm=k))
    out.append(LaunchOptions(order="longest_first"))
    out.append(LaunchOptions(order="row_major"))
    return out


def time_steps(batch: BatchedCV, steps: int, warmup: int = 1) -> float:
    """Mean device milliseconds per step (CUDA events on the current stream)."""
    batch.step(warmup)
    stream = torch.cuda.current_stream(batch.device)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(batch.device)
    a.record(stream)
    batch.step(steps)
    b.record(stream)
    torch.cuda.synchronize(batch.device)
    return a.elapsed_time(b) / steps


def autotune(jobs, candidates=None, steps: int = 3, refine: bool = True, use_cache: bool = True,
             margin: float = 0.015) -> LaunchOptions:
    """Launch options with the shortest step for this size mix, measured on
    copies of the jobs (the jobs themselves are not advanced).  A first
    one-knob sweep is followed, when ``refine``, by the combination of the
    best value of each knob.  Each candidate runs two untimed steps first, so
    that every job's cost-ordered hand-out reflects its current state.  The
    fastest candidate and the defaults are then timed again in turn, and the
    candidate replaces the defaults only when it is faster by more than
    ``margin`` over both rounds: a few steps per candidate are too few to tell
    apart options within a percent or two, and the defaults were chosen on
    long runs.  Results are cached per mix signature."""
    key = mix_signature(jobs)
    if use_cache and key in _TUNED:
        return _TUNED[key]
    cands = list(candidates) if candidates is not None else default_candidates()
    copies = [j.clone() for j in jobs]
    results = []

    def run(opt, record=True):
        b = BatchedCV(copies, options=opt, use_graph=True)
        try:
            ms = time_steps(b, steps, warmup=2)
        finally:
            b.close()
        if record:
            results.append((ms, opt))
        return ms

    for opt in cands:
        run(opt)
    base = LaunchOptions()
    if refine and candidates is None:
        best_of = {}
        for ms, opt in results:
            for f in ("batch", "blocks_per_sm", "defer", "order"):
                v = getattr(opt, f)
                if v != getattr(base, f) and (f not in best_of or ms < best_of[f][0]):
                    best_of[f] = (ms, v)
        base_ms = min(ms for ms, o in results if o == base)
        combo = LaunchOptions(**{f: v for f, (ms, v) in best_of.items() if ms < base_ms})
        if combo not in [o for _, o in results]:
            run(combo)
    best_ms, best = min(results, key=lambda r: r[0])
    if best != base and base in [o for _, o in results]:
        base_ms = min(ms for ms, o in results if o == base)
        again_best, again_base = run(best, record=False), run(base, record=False)
        if best_ms + again_best > (1.0 - margin) * (base_ms + again_base):
            best = base
    del copies
    _TUNED[key] = best
    return best


def tuning_report(jobs):
    """(ms, options) of every measured candidate of the cached mix, if any."""
    return _TUNED.get(mix_signature(jobs))


# --------------------------------------------------------------- size mixes
def cfg4_mix(n_jobs: int = 32, seed: int = 4, max_depth: int = 32):
    """The batched configuration's size mix: density grids from {16,32,64,128}^3,
    films from {64,128,256,512}^2, spp from {4,8,16}, depth 32 (seeded draw)."""
    rng = np.random.default_rng(seed)
    grids = rng.choice([16, 32, 64, 128], size=n_jobs)
    res = rng.choice([64, 128, 256, 512], size=n_jobs)
    spp = rng.choice([4, 8, 16], size=n_jobs)
    return [dict(grid=int(g), res=int(r), spp=int(s), max_depth=max_depth) for g, r, s in zip(grids, res, spp)]


def make_mix_jobs(mix, device="cuda", target_spp: int = 64, phase: str = "late", lr: float = 0.02,
                  keep_images: bool = False, seed_offset: int = 1000, supergrid: bool = False):
    """CVJob per entry of a size mix: Gaussian-blob medium of job seed
    seed_offset + j (constant albedo 0.8), target = the true grid rendered at
    target_spp, initial grid 0.8 x the true grid ('late') or constant 1.0
    ('early'), rr_depth = max_depth.  supergrid: each job's medium gets the
    majorant supergrid factor of scenes.majorant_factor_for."""
    from . import load_dict, scenes

    jobs = []
    for k, m in enumerate(mix):
        dens = scenes.blob_density(m["grid"], seed_offset + k)
        scene = load_dict(scenes.scene_dict(dens, 0.8, res=m["res"]), device=device)
        base = load_dict({"type": "prbvolpath", "max_depth": m["max_depth"], "rr_depth": m["max_depth"]})
        target = base.render(scene, 0, seed=17843 + k, spp=target_spp)
        init = (0.8 * dens) if phase == "late" else np.full_like(dens, 1.0)
        factor = scenes.majorant_factor_for(dens.shape[:3]) if supergrid else 0
        jobs.append(CVJob(init, 0.8, target, scene.sensors()[0], spp=m["spp"], max_depth=m["max_depth"],
                          rr_depth=m["max_depth"], seed=seed_offset * 7 + k * 1000, lr=lr, density_bounds=(0.0, 250.0),
                          keep_images=keep_images, majorant_factor=factor, device=device))
        del scene
    return jobs


def mix_paths(mix) -> int:
    return sum(m["res"] * m["res"] * 2 * m["spp"] for m in mix)

