"""Recursive control variate integrators: ``cv`` (plugins/cv_integrator.py)
and ``meta`` (plugins/metaintegrator.py).

Per step (cv_ps, plugins/cv_integrator.py:47-77): render (H, F) with the
nested two-state integrator, then on the GPU in one elementwise kernel
(rcv_cv_step): update the control weight from the EMA-Welford statistics when
``it > warmup``, blend ``img = w_s (img - H) + F`` and update the statistics
when ``it > 0``.  The adjoint is delegated to ``adjoint_integrator``.
"""
from __future__ import annotations

import ctypes as C

import torch

from .. import _lib
from ..core import Properties
from ..utils import stream_handle
from .twostatevolpath import TwoStatePRBVolpathIntegrator
from .welford import StatisticsEstimator


def _twostate_types():
    from .twostatepath import TwoStatePRBIntegrator

    return (TwoStatePRBIntegrator, TwoStatePRBVolpathIntegrator)


class _CVState:
    """Device buffers of the control variate: img, w_s, v_n plus the
    statistics (all zero-initialised like the reference's scalar zeros)."""

    def __init__(self, beta1: float, beta2: float):
        self.stats = StatisticsEstimator(beta1, beta2)
        self.img = self.w_s = self.v_n = None
        self.H = self.F = None

    def ensure(self, like: torch.Tensor) -> None:
        if self.img is None or self.img.shape != like.shape:
            self.img, self.w_s, self.v_n = (torch.zeros_like(like) for _ in range(3))
            self.stats._ensure(like)
            self.stats.n = 0

    def step(self, H: torch.Tensor, F: torch.Tensor, it: int, warmup: int, pre_update: bool) -> torch.Tensor:
        H = H.contiguous()
        F = F.contiguous()
        self.ensure(H)
        s = self.stats.state_struct(self.img, self.w_s, self.v_n)
        cnt = C.c_int32(self.stats.n)
        _lib.check(
            _lib.load().rcv_cv_step(
                C.byref(s), H.numel(), H.data_ptr(), F.data_ptr(), it, warmup, C.byref(cnt), self.stats.beta1,
                self.stats.beta2, int(pre_update), stream_handle(H.device),
            ),
            "rcv_cv_step",
        )
        self.stats.n = cnt.value
        self.H, self.F = H, F
        return self.img


class CVIntegrator:
    """``cv``: path-space recursive control variate around a two-state
    integrator (plugins/cv_integrator.py:9-94)."""

    def __init__(self, props: Properties):
        self.integrator = props.get("integrator")
        if type(self.integrator) not in _twostate_types():
            raise ValueError("CV integrator expects a 'twostate' integrator as nested integrator !")
        self.adjoint_integrator = props.get("adjoint_integrator", self.integrator)
        self.warmup = int(props.get("warmup", 1))
        self.beta1 = float(props.get("beta1", 0.9))
        self.beta2 = float(props.get("beta2", 0.999))
        self.reset()

    def reset(self):
        self.init = False

    def init_buffers(self):
        if self.init:
            return
        self.cv = _CVState(self.beta1, self.beta2)
        self.it = 0
        self.init = True

    # attributes of the reference (img, w_s, v_n, H, F, stats)
    @property
    def img(self):
        return self.cv.img

    @property
    def w_s(self):
        return self.cv.w_s

    @property
    def v_n(self):
        return self.cv.v_n

    @property
    def H(self):
        return self.cv.H

    @property
    def F(self):
        return self.cv.F

    @property
    def stats(self):
        return self.cv.stats

    def render(self, scene, sensor: int = 0, seed: int = 0, spp: int = 0, develop: bool = True, evaluate: bool = True):
        assert isinstance(sensor, int)
        self.init_buffers()
        H, F = self.integrator.render_twostates(scene, sensor, seed, spp)
        img = self.cv.step(H, F, self.it, self.warmup, False)
        self.it += 1
        return img.clone()

    def render_forward(self, scene, params, sensor=0, seed: int = 0, spp: int = 0, tangents=None):
        return self.adjoint_integrator.render_forward(scene, params, sensor, seed, spp, tangents=tangents)

    def render_backward(self, scene, params, grad_in, sensor=0, seed: int = 0, spp: int = 0):
        return self.adjoint_integrator.render_backward(scene, params, grad_in, sensor, seed, spp)

    def prefetch_adjoint(self, scene, sensor=0, seed: int = 0, spp: int = 0):
        pre = getattr(self.adjoint_integrator, "prefetch_adjoint", None)
        return pre(scene, sensor, seed, spp) if pre is not None else None


class MetaIntegrator:
    """``meta`` (plugins/metaintegrator.py:7-147): methods ``baseline``,
    ``cv_ps`` (path-space CV, two-state integrator) and ``cv_pss``
    (primary-sample-space CV from two single-state renders), with
    ``pre_update`` and ``force_baseline``.  The OptiX denoiser option of the
    reference is not available."""

    def __init__(self, props: Properties):
        self.denoise = bool(props.get("denoise", False))
        if self.denoise:
            raise ValueError("denoise=True needs the OptiX denoiser, which this implementation does not provide")
        self.force_baseline = bool(props.get("force_baseline", False))
        self.integrator = props.get("integrator")
        self.adjoint_integrator = props.get("adjoint_integrator", self.integrator)
        self.method = props.get("method", "baseline")
        if self.method not in ("baseline", "cv_ps", "cv_pss"):
            raise ValueError(f"unknown method '{self.method}'")
        if self.method == "cv_ps" and type(self.integrator) not in _twostate_types():
            raise ValueError("method 'cv_ps' expects a 'twostate' integrator as nested integrator")
        self.pre_update = bool(props.get("pre_update", False))
        self.warmup = int(props.get("warmup", 1))
        self.beta1 = float(props.get("beta1", 0.9))
        self.beta2 = float(props.get("beta2", 0.999))
        self.reset()

    def reset(self):
        self.init = False

    def init_buffers(self):
        if self.init:
            return
        self.img_ = None
        if "cv" not in self.method:
            return
        self.cv = _CVState(self.beta1, self.beta2)
        self.it = 0
        self.init = True

    @property
    def img(self):
        return self.cv.img if "cv" in self.method else self.img_

    def render(self, scene, sensor: int = 0, seed: int = 0, spp: int = 0, develop: bool = True, evaluate: bool = True):
        assert isinstance(sensor, int)
        self.init_buffers()
        img_noisy = None
        if self.method == "cv_ps":
            H, F = self.integrator.render_twostates(scene, sensor, seed, spp)
        else:
            img_noisy = self.integrator.render(scene, sensor, seed, spp, develop, evaluate)
        if self.method == "cv_pss":
            F = img_noisy
            H = self.cv.H if self.cv.H is not None else torch.zeros_like(F)
        if "cv" in self.method:
            img = self.cv.step(H, F, self.it, self.warmup, self.pre_update).clone()
            self.it += 1
        else:
            img = img_noisy
            self.img_ = img
        if self.method == "cv_pss":
            # re-render the current state with the next step's seed
            # (plugins/metaintegrator.py:117-119)
            self.cv.H = self.integrator.render(scene, sensor, seed + 1, spp, develop, evaluate)
        if self.force_baseline:
            if self.method != "cv_ps":
                return img_noisy
            return self.integrator.render(scene, sensor, seed, spp, develop, evaluate)
        return img

    def render_forward(self, scene, params, sensor=0, seed: int = 0, spp: int = 0, tangents=None):
        return self.adjoint_integrator.render_forward(scene, params, sensor, seed, spp, tangents=tangents)

    def render_backward(self, scene, params, grad_in, sensor=0, seed: int = 0, spp: int = 0):
        return self.adjoint_integrator.render_backward(scene, params, grad_in, sensor, seed, spp)

    def prefetch_adjoint(self, scene, sensor=0, seed: int = 0, spp: int = 0):
        pre = getattr(self.adjoint_integrator, "prefetch_adjoint", None)
        return pre(scene, sensor, seed, spp) if pre is not None else None
