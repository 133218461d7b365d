"""``render(scene, params, integrator, seed, spp, spp_grad)``: the
differentiable render entry point (``mi.render`` of the reference path and
``two_state_render``, plugins/twostatepath.py:10-95).

The forward pass calls ``integrator.render``; the backward pass calls
``integrator.render_backward`` with ``seed_grad`` / ``spp_grad`` and hands the
returned gradients to torch autograd, so ``loss.backward()`` accumulates them
into the optimizer's tensors (the ``dr.backward(loss)`` of optimize.py:122).
No AD tape is recorded: the adjoint replays paths from their seed.
"""
from __future__ import annotations

import torch

from . import _lib


class _RenderJob:
    __slots__ = ("scene", "params", "integrator", "sensor", "seed", "seed_grad", "spp", "spp_grad", "keys")


class _RenderOp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, job: _RenderJob, *tensors):
        ctx.job = job
        ctx.shapes = [t.shape for t in tensors]
        with torch.no_grad():
            # the adjoint's radiance pass needs only the parameters and the
            # gradient seed: it runs on a side stream beside the primal
            # render, and the backward pass then only replays
            pre = getattr(job.integrator, "prefetch_adjoint", None)
            launch = pre(job.scene, job.sensor, job.seed_grad, job.spp_grad) if pre is not None else None
            img = job.integrator.render(job.scene, job.sensor, job.seed, job.spp)
            if launch is not None:
                launch()
        return img

    @staticmethod
    def jvp(ctx, _job_tangent, *tangents):
        """Forward mode (torch.func.jvp / torch.autograd.forward_ad): the
        image derivative along the parameter tangents, from
        ``integrator.render_forward`` with the gradient seed and spp."""
        job = ctx.job
        tan = {k: t for k, t in zip(job.keys, tangents) if t is not None}
        return job.integrator.render_forward(job.scene, job.params, job.sensor, job.seed_grad, job.spp_grad,
                                             tangents=tan)

    @staticmethod
    def backward(ctx, grad_img):
        job = ctx.job
        grads = job.integrator.render_backward(
            job.scene, job.params, grad_img.contiguous(), job.sensor, job.seed_grad, job.spp_grad
        )
        out = [None]
        for key, shape in zip(job.keys, ctx.shapes):
            g = grads.get(key)
            out.append(None if g is None else g.reshape(shape))
        return tuple(out)


def default_seed_grad(seed: int) -> int:
    """``mi.sample_tea_32(seed, 1)[0]`` (plugins/twostatepath.py:87-89)."""
    return _lib.sample_tea_32(seed, 1)[0]


def render(scene, params=None, integrator=None, sensor: int = 0, seed: int = 0, seed_grad: int = 0, spp: int = 0,
           spp_grad: int = 0) -> torch.Tensor:
    if integrator is None:
        raise ValueError("render() needs an integrator")
    if params is not None and not hasattr(params, "differentiable"):
        raise Exception("params should be an instance of SceneParameters!")
    if spp_grad == 0:
        spp_grad = spp
    if seed_grad == 0:
        seed_grad = default_seed_grad(seed)
    elif seed_grad == seed:
        raise Exception(
            "The primal and differential seed should be different to ensure unbiased gradient computation!"
        )
    job = _RenderJob()
    job.scene, job.params, job.integrator, job.sensor = scene, params, integrator, sensor
    job.seed, job.seed_grad, job.spp, job.spp_grad = int(seed), int(seed_grad), int(spp), int(spp_grad)
    diff = params.differentiable() if params is not None else {}
    job.keys = list(diff.keys())
    tensors = [diff[k] for k in job.keys]
    if not tensors or not torch.is_grad_enabled():
        with torch.no_grad():
            return integrator.render(scene, sensor, job.seed, job.spp)
    return _RenderOp.apply(job, *tensors)
