#!/usr/bin/env python
"""Gradient-step throughput of the recursive-control-variate step on GB300.

Workload (default ``cfg2``): 64^3 density + 64^3 RGB albedo Gaussian-blob
medium, 512x512 film, spp = spp_grad = 16, max_depth = rr_depth = 64, cv_ps
with the two-state tracer, L2 loss against a 256-spp target of the true grid,
path-replay adjoint into density and albedo, Adam (lr 0.02) with clamping.
One step = params.update (state rotation) + two-state render + CV blend +
loss + adjoint + Adam; paths/step = H*W*(spp + spp_grad).

Prints ONE JSON line (rank 0).  ``--impl reference`` times the CPU
restatement of the same step on the host cores instead (the reference's own
llvm_ad_rgb path needs Mitsuba 3 / Dr.Jit, which are not available).

Multi-GPU: the step does not shard without an all-reduce of the gradient
grid, so N>1 runs N independent replicas (one job per rank, weak scaling, no
collective in the data path); value = all ranks' paths / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

METRIC = "gradient-step paths/s at matched gradient variance; p50/p99 step latency"
UNIT = "paths/s"
L2_BYTES = 129 * 2**20
FLUSH_BYTES = 512 * 2**20


# ------------------------------------------------------------------ helpers
def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def init_dist(backend: str):
    import torch.distributed as dist

    rank, world, _ = dist_info()
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist if world > 1 else None


def reduce_max(value: float, dist, device=None) -> float:
    """Max over ranks (identity without a process group)."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(value: float, dist, device=None) -> float:
    if dist is None:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def replica_seed(rank: int) -> int:
    """Per-rank job seed of a replica (rank 0 = the single-GPU job)."""
    return 1000 * rank


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
        except Exception:
            pass
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_figures(kernel: str, workload: str = "cfg2") -> dict:
    """Per-launch figures of `kernel` recorded from ncu captures in
    profiles/*.md (lines `<figure>[<kernel>]: <value>`, e.g.
    traffic_bytes_per_launch, l1_throughput_pct_128px, threads_per_inst).  A
    file counts only if its `workload:` line names the bench's workload and
    its `source_digest:` line matches the digest of the current CUDA
    sources; otherwise its figures are left out."""
    from recursive_control_variates_gb300 import _build

    cur = _build.source_digest()
    figures, stale = {}, []
    for f in sorted((ROOT / "profiles").glob("*.md")):
        txt = f.read_text()
        found = re.findall(rf"^(\w+)\[{re.escape(kernel)}\]:\s*([0-9.eE+-]+)\s*$", txt, re.M)
        if not found:
            continue
        w = re.search(r"^workload:\s*(\S+)\s*$", txt, re.M)
        if w is None or w.group(1) != workload:
            continue
        m = re.search(r"^source_digest:\s*([0-9a-f]+)\s*$", txt, re.M)
        if m is None or m.group(1) != cur:
            stale.append(f"{f.name} ({m.group(1) if m else 'no digest'})")
            continue
        for k, v in found:
            figures.setdefault(k, float(v))
    return {"figures": figures, "source_digest": cur, "stale": stale}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, interval_ms: int = 50):
        self.gpu = gpu_index
        self.interval_ms = int(interval_ms)
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", str(self.interval_ms),
                 "-i", str(self.gpu)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        rows = []
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, flags in rows for i, f in enumerate(flags) if f.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# --------------------------------------------------------------- workload
def initial_density(cfg, true_density, phase: str):
    """Starting grid of the timed job.  'late': 0.8 x the true grid, the
    converging phase the recursive control variate is designed for (the
    medium is as dense as the configuration's medium family); 'early': the
    constant grid of the configuration's optimisation start (cfg.init)."""
    if phase == "late":
        return (0.8 * true_density).astype(np.float32)
    if phase == "early":
        return np.full_like(true_density, cfg.init)
    raise ValueError(f"unknown phase {phase!r}")


class Job:
    """One optimisation job of the configuration, resident on the device."""

    def __init__(self, cfg, device, seed: int, phase: str = "late", target=None, majorant_factor: int = 0,
                 pair: bool = True):
        import torch

        import recursive_control_variates_gb300 as rcv
        from recursive_control_variates_gb300 import scenes

        self.rcv, self.scenes, self.cfg, self.device, self.seed = rcv, scenes, cfg, device, seed
        dens, alb = scenes.config_grids(cfg)
        self.true_density, self.true_albedo = dens, alb
        if target is None:
            scene_ref = rcv.load_dict(scenes.scene_dict(dens, alb, res=cfg.res), device=device)
            base = rcv.load_dict({"type": "prbvolpath", "max_depth": cfg.max_depth, "rr_depth": cfg.max_depth})
            target = base.render(scene_ref, 0, seed=17843, spp=cfg.spp_ref).contiguous()
            del scene_ref
        self.target = target
        self.init_density = initial_density(cfg, dens, phase)
        self.has_albedo = not np.isscalar(alb)
        self.init_albedo = np.full_like(alb, 0.5) if self.has_albedo else alb
        self.scene = rcv.load_dict(scenes.scene_dict(self.init_density, self.init_albedo, res=cfg.res), device=device)
        if majorant_factor:
            self.scene.named_shapes()["object"].interior_medium().set_majorant_resolution_factor(majorant_factor)
        self.params = rcv.traverse(self.scene)
        self.integrator = rcv.load_dict({
            "type": "cv",
            "integrator": {"type": "twostateprbvolpath", "max_depth": cfg.max_depth, "rr_depth": cfg.max_depth,
                           "pair_adjoint": pair},
        })
        self.opt = rcv.ad.Adam(lr=cfg.lr)
        self.opt[scenes.DENSITY_KEY] = self.init_density
        self.opt.set_bounds(scenes.DENSITY_KEY, *cfg.clamp)
        if self.has_albedo:
            self.opt[scenes.ALBEDO_KEY] = self.init_albedo
            self.opt.set_bounds(scenes.ALBEDO_KEY, 0.0, 1.0)
        # twice, so that old = new = initial state (utils.py:62-66)
        self.params.update(self.opt)
        self.params.update(self.opt)
        self.it = 0
        self.torch = torch

    def step(self, target=None, before_loss=None):
        rcv = self.rcv
        self.params.update(self.opt)
        img = rcv.render(self.scene, self.params, integrator=self.integrator, seed=self.seed + self.it,
                         spp=self.cfg.spp, spp_grad=self.cfg.spp_grad)
        if before_loss is not None:
            before_loss()
        loss = rcv.l2_loss(img, self.target if target is None else target)
        loss.backward()
        self.opt.step()
        self.it += 1
        return loss

    def counters(self):
        return self.integrator.integrator.counters(self.device).clone()

    def paths_per_step(self) -> int:
        return self.cfg.paths_per_step()


def workload_name(cfg, has_albedo: bool) -> str:
    """The workload string of both arms' JSON lines."""
    alb = f" + {cfg.grid}^3 RGB albedo" if has_albedo else f", albedo {cfg.albedo}"
    return (f"{cfg.name}: {cfg.grid}^3 density{alb}, {cfg.res}x{cfg.res}, spp={cfg.spp}, spp_grad={cfg.spp_grad}, "
            f"max_depth={cfg.max_depth}, cv_ps + path-replay adjoint + Adam")


def algorithmic_bytes(cfg, has_albedo: bool, c_two, c_adj, tape: bool = True) -> dict:
    """Algorithmic bytes per launch of the two tracer kernels from the device
    counters (lookups, scatters, gradient events) of one step.

    Two-state pass: 64 B per density lookup (8 corners x 2 states), 192 B of
    albedo per real scattering event, 24 B of film per pixel.  Adjoint: 32 B
    per density lookup of its passes, 32 B per gradient reduction (8 corners),
    96 B of albedo read and 96 B reduced per scattering event, 12 B of dL per
    pixel.  Each gradient event counts a 32-B read and a 32-B reduction,
    whether the gradient pass reads the grid again (the replay's lookups,
    counted as lookups) or keeps the value beside the event (the tape); the
    tape itself (20 B written and read per event) is intermediate storage
    and not counted."""
    lookups2 = float(c_two[1] + c_two[2])
    scat2 = float(c_two[3])
    npix = cfg.res * cfg.res
    two = 64.0 * lookups2 + (192.0 * scat2 if has_albedo else 0.0) + 24.0 * npix
    lookups_a = float(c_adj[1] + c_adj[2])
    scat_a = float(c_adj[3])
    ge, ae = float(c_adj[4]), float(c_adj[5])
    per_event = 32.0 + (32.0 if tape else 0.0)
    albedo = 96.0 * scat_a + (96.0 + 96.0 if tape else 96.0) * ae
    adj = 32.0 * lookups_a + per_event * ge + (albedo if has_albedo else 0.0) + 12.0 * npix
    return {"trace_twostate": two, "trace_adjoint": adj}


def run_ours(args, cfg):
    import torch

    import recursive_control_variates_gb300 as rcv
    from recursive_control_variates_gb300 import profiling

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    dist = init_dist("nccl")
    lib = rcv.load_library()
    job = Job(cfg, device, seed=replica_seed(rank), pair=not args.no_pair)
    paths = job.paths_per_step()
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device)

    for _ in range(args.warmup):
        job.step()
    torch.cuda.synchronize()

    # ------------------------------------------------- device-timed region
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = lib.rcv_kernel_launches()
    timer = profiling.KernelTimer()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks, timer:
        for i in range(args.steps):
            flush.fill_(float(i))  # evict the previous step from L2 (> 129 MB)
            starts[i].record(stream)
            job.step()
            ends[i].record(stream)
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    launches = lib.rcv_kernel_launches() - launches0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    local_total_s = sum(step_ms) / 1e3
    total_s = reduce_max(local_total_s, dist, device)
    ms_per_step = total_s * 1e3 / args.steps
    value = paths * world * args.steps / total_s
    kern = timer.summary()

    # roofline of the dominant kernel.  In the timed steps the adjoint's
    # radiance pass runs on a side stream beside the two-state pass, so their
    # launch durations overlap; the per-kernel durations come from a few more
    # steps with the two passes one after the other (same kernels, same
    # inputs), each launch alone on the GPU.
    inner = job.integrator.integrator
    inner.overlap_adjoint = False
    serial = profiling.KernelTimer()
    with serial:
        for i in range(3):
            flush.fill_(float(i))
            job.step()
    inner.overlap_adjoint = True
    kern_serial = serial.summary()
    # the counters mix both tracers; split with a separate 1-step measurement
    c_two, c_adj = split_counters(job)
    delta = (c_two + c_adj).astype(np.float64)  # event counts of one step (counted separately)
    algo = algorithmic_bytes(cfg, job.has_albedo, c_two, c_adj, tape=job.integrator.integrator.adjoint == 0)
    dom = max(("trace_twostate", "trace_adjoint"), key=lambda k: kern_serial.get(k, {}).get("total_ms", 0.0))
    peaks = measured_peaks()
    dur_s = kern_serial[dom]["mean_ms"] / 1e3
    achieved = algo[dom] / dur_s / 1e9
    prof = profile_figures(dom, cfg.name)
    fig = prof["figures"]
    roof = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
            "peak_source": peaks["source"], "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
            "traffic": fig.get("traffic_bytes_per_launch"), "algorithmic_bytes_per_launch": algo[dom],
            "mean_launch_ms": round(kern_serial[dom]["mean_ms"], 4),
            "timing": "launches timed alone (3 steps without the side-stream overlap)",
            # the ceiling the tracer launches actually meet (grids are L2-resident):
            # L1 throughput and lanes per warp instruction from the same capture
            "threads_per_inst": fig.get("threads_per_inst"),
            "l1_throughput_pct_128px": fig.get("l1_throughput_pct_128px"),
            "profile_note": ("traffic and threads_per_inst: 1-pass ncu metrics of this launch size; "
                             "l1_throughput_pct_128px: the same medium at a 128^2 film (a multi-pass metric, "
                             "captured on the small case only)"),
            "profile_source_digest": prof["source_digest"]}
    if not fig:
        roof["profile_note"] = (f"no ncu summary in profiles/ was captured for {cfg.name} from the current CUDA sources"
                                + (f"; stale: {', '.join(prof['stale'])}" if prof["stale"] else ""))

    # --------------------------------------------------- end-to-end (API)
    e2e = None
    if not args.no_e2e:
        target_host = job.target.cpu().pin_memory()
        for _ in range(2):
            job.step(target_host.to(device, non_blocking=True)).item()
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()
        # each step copies its target from pinned host memory on a copy
        # stream, overlapped with the render (the loss waits for the copy),
        # and copies its loss into pinned host memory; the host reads step
        # i's loss while step i+1 runs, as a training loop that logs its loss
        # does, so the launches of a step are issued during the previous one
        copy_stream = torch.cuda.Stream(device)
        tgts = [torch.empty_like(job.target) for _ in range(2)]
        consumed = [None, None]  # main-stream event after the loss read tgts[k]
        loss_host = torch.empty(args.steps, dtype=torch.float32).pin_memory()
        losses = []
        main = torch.cuda.current_stream(device)
        pending = None  # (step, event after its loss copy)
        t0 = time.perf_counter()
        for i in range(args.steps):
            k = i & 1
            with torch.cuda.stream(copy_stream):
                if consumed[k] is not None:
                    copy_stream.wait_event(consumed[k])
                tgts[k].copy_(target_host, non_blocking=True)
                copied = torch.cuda.Event()
                copied.record(copy_stream)
            loss = job.step(tgts[k], before_loss=lambda: main.wait_event(copied))
            consumed[k] = torch.cuda.Event()
            consumed[k].record(main)
            loss_host[i].copy_(loss.detach(), non_blocking=True)
            done = torch.cuda.Event()
            done.record(main)
            if pending is not None:
                pending[1].synchronize()
                losses.append(float(loss_host[pending[0]]))
            pending = (i, done)
        pending[1].synchronize()
        losses.append(float(loss_host[pending[0]]))
        torch.cuda.synchronize()
        assert len(losses) == args.steps and all(math.isfinite(v) for v in losses)
        el = reduce_max(time.perf_counter() - t0, dist, device)
        e2e = {"value": paths * world * args.steps / el, "unit": UNIT,
               "h2d_bytes_per_step": int(target_host.numel() * 4), "d2h_bytes_per_step": 4,
               "ms_per_step": el * 1e3 / args.steps}

    early = None
    if not args.no_early:
        early = time_phase(args, cfg, device, dist, job.target, "early", world, flush)
    supergrid = None
    if args.majorant_factor > 0:
        supergrid = time_phase(args, cfg, device, dist, job.target, "late", world, flush,
                               majorant_factor=args.majorant_factor)
    sparse = None
    if args.majorant_factor > 0 and not args.no_sparse:
        # a medium sparse enough for the supergrid: one blob in a 128^3 grid
        from recursive_control_variates_gb300 import scenes as _sc

        scfg = _sc.CONFIGS["sparse128"]
        glob = time_phase(args, scfg, device, dist, None, "late", world, flush)
        sg = time_phase(args, scfg, device, dist, None, "late", world, flush, majorant_factor=8)
        sparse = {"workload": "sparse128: one Gaussian blob in a 128^3 grid, 512^2, spp 16, depth 64, albedo 0.8",
                  "global": glob, "supergrid": sg, "supergrid_speedup": glob["ms_per_step"] / sg["ms_per_step"]}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(cfg, job, target_seconds=args.cpu_seconds)

    has_albedo = job.has_albedo
    del job
    torch.cuda.empty_cache()
    surface = None if args.no_surface else surface_form(args, device, dist, world, flush)
    # the batched and served forms run on a single GPU only (rank 0 of one)
    batched = None if (args.no_batched or world > 1) else batched_form(args, device, flush)
    served = None if (args.no_served or world > 1) else served_form(args, device)

    ms_sorted = sorted(step_ms)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Gaussian-blob medium; no public dataset)",
        "config": {"workload": workload_name(cfg, has_albedo), "paths_per_step": paths, "parallelism": f"replicas x{world}",
                   "l2": "flushed between timed steps (512 MB write)",
                   "tracers": ("two-state render and adjoint radiance pass in one persistent launch"
                               if not args.no_pair else "two-state render and adjoint radiance pass on two streams")},
        "p50_ms": ms_sorted[len(ms_sorted) // 2],
        "p99_ms": ms_sorted[min(len(ms_sorted) - 1, int(math.ceil(0.99 * len(ms_sorted))) - 1)],
        "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
        "kernels": {k: {"launches": v["launches"], "mean_ms": round(v["mean_ms"], 4)} for k, v in kern.items()},
        "kernels_alone": {k: {"launches": v["launches"], "mean_ms": round(v["mean_ms"], 4)}
                          for k, v in kern_serial.items()},
        "counters_per_step": {"paths": float(delta[0]), "lookups": float(delta[1]), "nee_lookups": float(delta[2]),
                              "scatters": float(delta[3]), "grad_events": float(delta[4])},
        "clocks": clocks.summary(),
        "phase": "late (density starts at 0.8 x the true grid)",
        "early_phase": early,
        "supergrid": supergrid,
        "supergrid_sparse": sparse,
        "surface": surface,
        "batched": batched,
        "served": served,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def surface_form(args, device, dist, world, flush):
    """cfg3: the two-state surface tracer (`twostateprb`) step on a 1024^2
    film (ground plane with a 512^2 RGB texture, 3 spheres, an area light),
    spp 8, depth 8, through the plain API; device-timed steps."""
    import torch

    import recursive_control_variates_gb300 as rcv
    from recursive_control_variates_gb300 import scenes

    cfg = scenes.SURFACE_CONFIGS["cfg3"]
    true_tex = scenes.value_noise(cfg.tex_res, 7)
    ref_scene = rcv.load_dict(scenes.surface_scene_dict(true_tex, cfg.res), device=device)
    base = rcv.load_dict({"type": "twostateprb", "max_depth": cfg.max_depth, "rr_depth": cfg.rr_depth})
    target = base.render(ref_scene, 0, seed=17843, spp=64).contiguous()
    del ref_scene
    init = np.full_like(true_tex, cfg.init)
    scene = rcv.load_dict(scenes.surface_scene_dict(init, cfg.res), device=device)
    params = rcv.traverse(scene)
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprb", "max_depth": cfg.max_depth,
                                                         "rr_depth": cfg.rr_depth}})
    opt = rcv.ad.Adam(lr=cfg.lr)
    opt[scenes.TEXTURE_KEY] = init
    opt.set_bounds(scenes.TEXTURE_KEY, 0.0, 1.0)
    params.update(opt)
    params.update(opt)
    it = [0]

    def step():
        params.update(opt)
        img = rcv.render(scene, params, integrator=integ, seed=replica_seed(dist_info()[0]) + it[0], spp=cfg.spp)
        rcv.l2_loss(img, target).backward()
        opt.step()
        it[0] += 1

    for _ in range(args.warmup):
        step()
    stream = torch.cuda.current_stream(device)
    steps = max(args.steps // 4, 10)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for i, (a, b) in enumerate(ev):
        flush.fill_(float(i))
        a.record(stream)
        step()
        b.record(stream)
    torch.cuda.synchronize()
    ms = sorted(a.elapsed_time(b) for a, b in ev)
    total = reduce_max(sum(ms) / 1e3, dist, device)
    paths = cfg.paths_per_step()
    cpu = None
    if dist_info()[0] == 0 and world == 1 and not args.no_cpu_baseline:
        # the texture state of the last step on the CPU restatement
        bsdf = scene.named_shapes()["plane"].bsdf
        cpu = surface_cpu_baseline(cfg, bsdf.old.texture.data.cpu().numpy(), bsdf.new.texture.data.cpu().numpy())
    return {"workload": f"cfg3: {cfg.res}^2 two-state surface scene (plane + {cfg.tex_res}^2 RGB texture, 3 spheres, "
                        f"area light), spp={cfg.spp}, spp_grad={cfg.spp_grad}, max_depth={cfg.max_depth}, cv_ps",
            "value": paths * world * steps / total, "unit": UNIT, "ms_per_step": total * 1e3 / steps, "steps": steps,
            "p50_ms": pctl(ms, 0.5), "p99_ms": pctl(ms, 0.99), "paths_per_step": paths, "cpu_baseline": cpu}


def time_phase(args, cfg, device, dist, target, phase, world, flush, majorant_factor=0):
    """Device-timed steps of a second job started in another phase (or with
    a majorant supergrid)."""
    import torch

    job = Job(cfg, device, seed=replica_seed(dist_info()[0]) + 77, phase=phase, target=target,
              majorant_factor=majorant_factor, pair=not args.no_pair)
    for _ in range(args.warmup):
        job.step()
    stream = torch.cuda.current_stream(device)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize()
    for i, (a, b) in enumerate(ev):
        flush.fill_(float(i))
        a.record(stream)
        job.step()
        b.record(stream)
    torch.cuda.synchronize()
    total = reduce_max(sum(a.elapsed_time(b) for a, b in ev) / 1e3, dist, device)
    c_two, c_adj = split_counters(job)
    d = (c_two + c_adj).astype(np.float64)
    paths = job.paths_per_step()
    return {"value": paths * world * args.steps / total, "unit": UNIT, "ms_per_step": total * 1e3 / args.steps,
            "start": f"density {'constant ' + str(cfg.init) if phase == 'early' else '0.8 x true grid'}",
            "majorant": f"supergrid, factor {majorant_factor}" if majorant_factor else "global",
            "lookups_per_path": float((d[1] + d[2]) / max(d[0], 1.0))}


def split_counters(job):
    """Per-kernel counters of one extra (untimed) step, with the counting
    tracer variants."""
    import torch

    integ = job.integrator.integrator
    integ.count_events = True
    cnt = integ.counters(job.device)
    job.params.update(job.opt)
    before = cnt.clone()
    H, F = integ.render_twostates(job.scene, 0, seed=job.seed + 10**6, spp=job.cfg.spp)
    mid = cnt.clone()
    g = torch.ones_like(job.target) / job.target.numel()
    integ.render_backward(job.scene, job.params, g, 0, seed=job.seed + 2 * 10**6, spp=job.cfg.spp_grad)
    after = cnt.clone()
    torch.cuda.synchronize()
    integ.count_events = False
    return (mid - before).cpu().numpy(), (after - mid).cpu().numpy()


# ------------------------------------------------------------ CPU baseline
# ------------------------------------------------- batched and served forms
def pctl(values, q):
    v = sorted(values)
    return v[min(len(v) - 1, max(0, int(math.ceil(q * len(v))) - 1))]


def plain_mix_setup(mix, jobs, device):
    """The plain single-job API objects of each job of a mix, at the job's
    current parameters (load_dict / traverse / cv integrator / ad.Adam)."""
    import recursive_control_variates_gb300 as rcv
    from recursive_control_variates_gb300 import scenes

    plains = []
    for m, job in zip(mix, jobs):
        dens0 = job.params().detach().cpu().numpy()[..., None]
        scene = rcv.load_dict(scenes.scene_dict(dens0, 0.8, res=m["res"], spp=m["spp"]), device=device)
        params = rcv.traverse(scene)
        integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath",
                                                             "max_depth": m["max_depth"], "rr_depth": m["max_depth"]}})
        opt = rcv.ad.Adam(lr=0.02)
        opt[scenes.DENSITY_KEY] = dens0
        opt.set_bounds(scenes.DENSITY_KEY, 0.0, 250.0)
        params.update(opt)
        params.update(opt)
        plains.append([scene, params, integ, opt, job.target, job.seed, m["spp"], 0])
    return plains


def plain_mix_step(plains):
    import recursive_control_variates_gb300 as rcv

    for p in plains:
        scene, params, integ, opt, target, seed, spp, it = p
        params.update(opt)
        img = rcv.render(scene, params, integrator=integ, seed=seed + it, spp=spp)
        rcv.l2_loss(img, target).backward()
        opt.step()
        p[7] += 1


def batched_form(args, device, flush):
    """cfg4: 32 uneven cv_ps jobs advanced by one BatchedCV step per
    iteration (CUDA graph, autotuned launch options), against the plain
    single-job API stepping the same jobs one after another."""
    import torch

    from recursive_control_variates_gb300 import batch

    mix = batch.cfg4_mix(32)[:args.batched_jobs]
    jobs = batch.make_mix_jobs(mix, device=device, target_spp=args.target_spp)
    paths = sum(j.paths_per_step() for j in jobs)
    plains = plain_mix_setup(mix, jobs, device) if args.plain_rounds > 0 else None
    t0 = time.perf_counter()
    best = batch.autotune(jobs, steps=2) if not args.no_autotune else batch.LaunchOptions()
    best = dataclasses.replace(best, pair_tracers=not args.no_pair)
    tune_s = time.perf_counter() - t0
    b = batch.BatchedCV(jobs, options=best, use_graph=True)
    stream = torch.cuda.current_stream(device)
    b.step(args.warmup)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.batched_steps)]
    with ClockSampler(device.index or 0) as clocks:
        for i, (a, e) in enumerate(ev):
            flush.fill_(float(i))
            a.record(stream)
            b.step()
            e.record(stream)
        torch.cuda.synchronize()
    ms = [a.elapsed_time(e) for a, e in ev]
    b.close()
    # event counts of one more step, by the counting tracer variants
    bc = batch.BatchedCV(jobs, options=dataclasses.replace(best, count_events=True), use_graph=False)
    bc.step()
    torch.cuda.synchronize()
    dc = bc.counters().cpu().numpy().astype(np.float64)
    bc.close()
    total = sum(ms) / 1e3
    value = paths * len(ms) / total
    # the batched form per film size: the jobs of one film size in a batch of
    # their own (same launch options), so that its lead over the plain API
    # shows per size
    batched_by_film = {}
    for r in sorted({int(m["res"]) for m in mix}):
        sel = [j for m, j in zip(mix, jobs) if int(m["res"]) == r]
        bf = batch.BatchedCV(sel, options=best, use_graph=True)
        bf.step(2)
        torch.cuda.synchronize()
        evf = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(10)]
        for i, (a, e) in enumerate(evf):
            flush.fill_(float(i))
            a.record(stream)
            bf.step()
            e.record(stream)
        torch.cuda.synchronize()
        fms = sum(a.elapsed_time(e) for a, e in evf) / len(evf)
        pp = sum(int(j.paths_per_step()) for j in sel)
        batched_by_film[f"{r}x{r}"] = {"jobs": len(sel), "paths_per_step": pp, "ms": round(fms, 3),
                                       "paths_per_s": pp / (fms / 1e3)}
        bf.close()
    plain_value = plain_ms = plain_wall = plain_by_film = None
    if plains is not None:
        # plain single-job form: the same jobs through the single-job API.
        # Three untimed rounds: the first two steps of the first job pay
        # one-time host costs (kernels loaded on first launch) that the events
        # around a round would count when the form runs on its own.
        for _ in range(3):
            plain_mix_step(plains)
        torch.cuda.synchronize()
        rounds = args.plain_rounds
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        a.record(stream)
        for _ in range(rounds):
            plain_mix_step(plains)
        e.record(stream)
        torch.cuda.synchronize()
        plain_wall = (time.perf_counter() - t0) / rounds * 1e3
        plain_ms = a.elapsed_time(e) / rounds
        plain_value = paths / (plain_ms / 1e3)
        # one more round timed job by job: where the batched form's lead
        # comes from (small films cannot fill the GPU in a single-job launch)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in plains]
        for p, (pa, pe) in zip(plains, ev):
            pa.record(stream)
            plain_mix_step([p])
            pe.record(stream)
        torch.cuda.synchronize()
        by_film = {}
        for m, job, (pa, pe) in zip(mix, jobs, ev):
            g = by_film.setdefault(int(m["res"]), {"jobs": 0, "paths_per_step": 0, "ms": 0.0})
            g["jobs"] += 1
            g["paths_per_step"] += int(job.paths_per_step())
            g["ms"] += pa.elapsed_time(pe)
        plain_by_film = {f"{r}x{r}": dict(g, ms=round(g["ms"], 3), paths_per_s=g["paths_per_step"] / (g["ms"] / 1e3))
                         for r, g in sorted(by_film.items())}
    return {
        "workload": f"cfg4: {len(jobs)} cv_ps jobs, grids {{16,32,64,128}}^3, films {{64..512}}^2, spp {{4,8,16}}, "
                    "depth 32, constant albedo 0.8, one persistent launch per tracer pass, CUDA graph",
        "value": value, "unit": UNIT, "ms_per_step": total * 1e3 / len(ms), "steps": len(ms),
        "p50_ms": pctl(ms, 0.5), "p99_ms": pctl(ms, 0.99), "paths_per_step": paths,
        "launch_options": best.__dict__, "autotune_s": round(tune_s, 2), "clocks": clocks.summary(),
        "gpu_launches_per_step": b.kernels_per_step,
        "plain_value": plain_value, "plain_ms_per_round": plain_ms, "plain_wall_ms_per_round": plain_wall,
        "speedup_vs_plain": value / plain_value if plain_value else None,
        "plain_by_film": plain_by_film,
        "batched_by_film": batched_by_film,
        "lead_by_film": ({k: round(v["paths_per_s"] / plain_by_film[k]["paths_per_s"], 3)
                          for k, v in batched_by_film.items() if k in plain_by_film} if plain_by_film else None),
        "lookups_per_path": float((dc[0][1] + dc[0][2] + dc[1][1] + dc[1][2]) / max(dc[0][0] + dc[1][0], 1.0)),
        "l2": "flushed between timed steps (512 MB write)",
    }


def served_form(args, device):
    """cfg5: Poisson arrivals (2000 req/s) of gradient-step requests over 64
    resident cfg4-mix jobs + 8 jobs at 256^3 / 1024^2 / spp 16, continuous
    batching under a 120 GB HBM budget; p50/p99 request latency and paths/s."""
    import torch

    from recursive_control_variates_gb300 import batch, serve

    mix = serve.cfg5_mix()
    jobs = batch.make_mix_jobs(mix, device=device, target_spp=args.target_spp, seed_offset=5000)
    server = serve.StepServer(120 * 10**9, device=device, options=batch.autotune(jobs[:64], steps=1), pipeline=2)
    ids = [server.add_job(j) for j in jobs]
    resident = sum(server.is_resident(i) for i in ids)
    for i in ids:  # warm-up: one step of every job
        server.submit(i)
    server.drain()
    torch.cuda.synchronize()
    server.stats = serve.ServerStats()
    arrivals = serve.poisson_arrivals(2000.0, args.served_requests, ids, seed=11)
    t0 = time.perf_counter()
    reqs = server.run_arrivals(arrivals)
    wall = time.perf_counter() - t0
    lat = serve.latency_summary(reqs)
    paths = server.stats.paths
    # The configured 2000 req/s offers several times what the GPU serves, so
    # the latencies above grow with the number of requests (queueing).  The
    # same mix at 80 % of the measured throughput shows the serving latency.
    mean_paths = float(np.mean([j.paths_per_step() for j in jobs]))
    rate = 0.8 * (paths / wall) / mean_paths
    stats = server.stats  # of the configured run
    server.stats = serve.ServerStats()
    t1 = time.perf_counter()
    reqs80 = server.run_arrivals(serve.poisson_arrivals(rate, args.served_requests, ids, seed=12))
    wall80 = time.perf_counter() - t1
    lat80 = serve.latency_summary(reqs80)
    at80 = {"rate_req_s": round(rate, 1), "requests": len(reqs80), "value": server.stats.paths / wall80,
            "p50_ms": lat80["p50_ms"], "p99_ms": lat80["p99_ms"], "mean_ms": lat80["mean_ms"],
            "mean_jobs_per_tick": float(np.mean(server.stats.jobs_per_tick))}
    server.close()
    return {
        "workload": "cfg5: Poisson 2000 req/s over 64 cfg4-mix jobs + 8 jobs (256^3, 1024^2, spp 16, depth 32), "
                    "continuous batching, 120 GB HBM budget",
        "requests": len(reqs), "value": paths / wall, "unit": UNIT, "wall_s": wall,
        "p50_ms": lat["p50_ms"], "p99_ms": lat["p99_ms"], "mean_ms": lat["mean_ms"],
        "ticks": stats.ticks, "mean_jobs_per_tick": float(np.mean(stats.jobs_per_tick)),
        "plan_reuses": stats.plan_reuses, "resident_jobs": int(resident),
        "resident_gb": round(server.resident_bytes() / 1e9, 2),
        "offered_paths_per_s": 2000.0 * mean_paths,
        "at_80pct_of_served": at80,
    }


def oracle_step_factory(cfg, density_old, density_new, albedo_old, albedo_new, target, threads):
    """One CPU gradient step (two-state render + CV + loss + adjoint) on a
    band of image rows, with the C++ restatement of the path."""
    from oracle import oracle as O

    cam = O.camera_basis(cfg.res, cfg.res)
    has_alb = albedo_new is not None and not np.isscalar(albedo_new)
    sc = O.Scene(cam, density_old, density_new, albedo_old=albedo_old if has_alb else None,
                 albedo_new=albedo_new if has_alb else None,
                 albedo_const=albedo_new if not has_alb else 0.8, max_depth=cfg.max_depth)
    cv = O.CVOracle()

    def step(seed, rows):
        """rows = (first, end, stride): every stride-th row is traced."""
        H, F = O.render_twostates(sc, seed, cfg.spp, threads=threads, rows=rows)
        sel = slice(*rows)
        img = cv.step(H[sel], F[sel])
        g = np.zeros_like(H)
        g[sel] = 2.0 * (img - target[sel]) / target.size
        O.backward(sc, seed + 7, cfg.spp_grad, g, threads=threads, rows=rows)
        return len(range(*rows)) * cfg.res * (cfg.spp + cfg.spp_grad)

    return step, sc


def row_sample(res: int, step_fn, seconds: float):
    """Every-k-th-row sample of the image sized so that one step takes about
    `seconds` (rows spread over the whole image keep it representative)."""
    probe = (0, res, max(1, res // 8))
    t0 = time.perf_counter()
    step_fn(1, probe)
    per_row = (time.perf_counter() - t0) / len(range(*probe))
    nrows = int(min(res, max(4, seconds / max(per_row, 1e-6))))
    stride = max(1, res // nrows)
    return (stride // 2, res, stride)


def cpu_baseline(cfg, job, target_seconds: float = 15.0):
    """Oracle timed on a bounded band of rows of the same workload."""
    from oracle import oracle as O

    threads = O.default_threads()
    dens_new = job.scene.named_shapes()["object"].interior_medium().new.density.cpu().numpy()[..., 0]
    dens_old = job.scene.named_shapes()["object"].interior_medium().old.density.cpu().numpy()[..., 0]
    med = job.scene.named_shapes()["object"].interior_medium()
    alb_new = med.new.albedo_grid.cpu().numpy() if job.has_albedo else cfg.albedo
    alb_old = med.old.albedo_grid.cpu().numpy() if job.has_albedo else cfg.albedo
    target = job.target.cpu().numpy()
    step, _ = oracle_step_factory(cfg, dens_old, dens_new, alb_old, alb_new, target, threads)
    rows = row_sample(cfg.res, step, target_seconds)
    step, _ = oracle_step_factory(cfg, dens_old, dens_new, alb_old, alb_new, target, threads)
    t0 = time.perf_counter()
    n = step(2, rows)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"every {rows[2]}th row ({len(range(*rows))} rows) x {cfg.res} px x (spp {cfg.spp} + spp_grad "
                      f"{cfg.spp_grad}) of {cfg.name} at the job's current state, one CPU gradient step ({n} paths, "
                      f"{dt:.1f} s), C++ restatement built with `{oracle_flags()}`, {threads} threads",
            "cpu": cpu_model(), "flags": oracle_flags()}


def surface_cpu_baseline(cfg, tex_old, tex_new, target_seconds: float = 4.0):
    """The surface oracle (two-state render + texture adjoint of the same
    scene) timed on an every-k-th-row sample of the config-3 step."""
    from oracle import oracle as O

    from recursive_control_variates_gb300 import scenes

    threads = O.default_threads()
    cam = O.camera_basis(cfg.res, cfg.res, *scenes.SURFACE_CAMERA)
    sc = O.SurfaceScene(cam, tex_old, tex_new, scenes.surface_spheres(cfg.seed), (0.0, 3.0, 0.0), (0.5, 0.5),
                        (15.0, 15.0, 15.0), plane_half=2.0, max_depth=cfg.max_depth, rr_depth=cfg.rr_depth)
    grad = np.random.default_rng(5).normal(0.0, 1.0, (cfg.res, cfg.res, 3)).astype(np.float32)

    def step(seed, rows):
        O.surface_render_twostates(sc, seed, cfg.spp, threads=threads, rows=rows)
        O.surface_backward(sc, seed + 1, cfg.spp_grad, grad, threads=threads, rows=rows)
        return len(range(*rows)) * cfg.res * (cfg.spp + cfg.spp_grad)

    rows = row_sample(cfg.res, step, target_seconds)
    t0 = time.perf_counter()
    n = step(3, rows)
    dt = time.perf_counter() - t0
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"every {rows[2]}th row ({len(range(*rows))} rows) x {cfg.res} px x (spp {cfg.spp} + spp_grad "
                      f"{cfg.spp_grad}) of {cfg.name}: two-state render and texture adjoint ({n} paths, {dt:.1f} s), "
                      f"C++ restatement built with `{oracle_flags()}`, {threads} threads",
            "cpu": cpu_model(), "flags": oracle_flags()}


def oracle_flags() -> str:
    from oracle import build as oracle_build

    return oracle_build.flags_text()


def cpu_model() -> str:
    try:
        txt = Path("/proc/cpuinfo").read_text()
        for key in ("model name", "Model", "CPU part"):
            m = re.search(rf"^{key}\s*:\s*(.+)$", txt, re.M)
            if m:
                return m.group(1).strip()
    except OSError:
        pass
    import platform

    return platform.processor() or platform.machine()


def run_reference(args, cfg):
    """CPU arm: the C++ restatement of the step on the host cores (the
    reference's own llvm_ad_rgb path needs Mitsuba 3 / Dr.Jit, absent here)."""
    from oracle import oracle as O
    from recursive_control_variates_gb300 import scenes

    rank, world, _ = dist_info()
    if rank != 0:
        return
    threads = O.default_threads()
    dens, alb = scenes.config_grids(cfg)
    has_alb = not np.isscalar(alb)
    init_d = initial_density(cfg, dens, "late")[..., 0]
    init_a = np.full_like(alb, 0.5) if has_alb else alb
    cam = O.camera_basis(cfg.res, cfg.res)
    ref_sc = O.Scene(cam, dens[..., 0], dens[..., 0], albedo_old=alb if has_alb else None,
                     albedo_new=alb if has_alb else None, albedo_const=alb if not has_alb else 0.8,
                     max_depth=cfg.max_depth)
    # every k-th row, k chosen so that one step takes ~args.cpu_step_seconds;
    # the states are the initial grid and the grid one Adam step later
    new_d = init_d + np.float32(cfg.lr)
    probe_target = O.render(ref_sc, 17843, cfg.spp, threads=threads, rows=(0, cfg.res, max(1, cfg.res // 8)))
    step, _ = oracle_step_factory(cfg, init_d, new_d, init_a, init_a, probe_target, threads)
    band = row_sample(cfg.res, step, args.cpu_step_seconds)
    target = O.render(ref_sc, 17843, cfg.spp_ref, threads=threads, rows=band)
    step, _ = oracle_step_factory(cfg, init_d, new_d, init_a, init_a, target, threads)
    times, npaths = [], 0
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        n = step(100 + i, band)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
            npaths = n
    total = sum(times)
    value = npaths * len(times) / total
    ts = sorted(times)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total * 1e3 / len(times), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded Gaussian-blob medium; no public dataset)", "impl": "reference",
        "config": {"workload": workload_name(cfg, has_alb), "paths_per_step": npaths,
                   "sample": f"every {band[2]}th row of {cfg.res} (the CPU step's row sample)"},
        "p50_ms": ts[len(ts) // 2] * 1e3, "p99_ms": ts[-1] * 1e3,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{len(range(*band))} rows x {cfg.res} px x (spp {cfg.spp} + spp_grad "
                                   f"{cfg.spp_grad}) per step; C++ restatement of the reference's path built "
                                   f"with `{oracle_flags()}` (its llvm_ad_rgb path needs Mitsuba 3 / Dr.Jit, not "
                                   f"installable offline)",
                         "cpu": cpu_model(), "flags": oracle_flags()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    # p50/p99 over >= 200 steps after >= 16 warm-up steps (optimize.py:105)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=16)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="cfg2")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-early", action="store_true", help="skip the early-phase measurement")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cpu-step-seconds", type=float, default=4.0)
    ap.add_argument("--no-batched", action="store_true", help="skip the batched (cfg4) form")
    ap.add_argument("--no-surface", action="store_true", help="skip the surface-scene (cfg3) step")
    ap.add_argument("--no-served", action="store_true", help="skip the served (cfg5) form")
    ap.add_argument("--form", choices=["all", "batched", "served"], default="all",
                    help="all: the headline line (plain cfg2) with the batched and served forms; batched / served: "
                         "only that form, printed as its own JSON object (profiling runs)")
    ap.add_argument("--batched-jobs", type=int, default=32)
    ap.add_argument("--no-sparse", action="store_true", help="skip the sparse-medium supergrid comparison")
    ap.add_argument("--majorant-factor", type=int, default=8,
                    help="also time the headline step with a majorant supergrid of this factor (0 = skip)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-pair", action="store_true",
                    help="run the adjoint's radiance pass on a side stream instead of in the two-state launch")
    ap.add_argument("--batched-steps", type=int, default=200)
    ap.add_argument("--plain-rounds", type=int, default=2)
    ap.add_argument("--served-requests", type=int, default=400)
    ap.add_argument("--target-spp", type=int, default=64, help="spp of the batched/served jobs' target renders")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    from recursive_control_variates_gb300 import scenes

    cfg = scenes.CONFIGS[args.config]
    if args.impl == "reference":
        run_reference(args, cfg)
    elif args.form != "all":
        run_form(args)
    else:
        run_ours(args, cfg)


def run_form(args):
    """One of the batched / served forms alone (single GPU)."""
    import torch

    torch.cuda.set_device(0)
    device = torch.device("cuda", 0)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device=device)
    out = batched_form(args, device, flush) if args.form == "batched" else served_form(args, device)
    print(json.dumps({"form": args.form, **out}), flush=True)


if __name__ == "__main__":
    main()
