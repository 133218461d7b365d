"""Small host utilities: CUDA stream handles and the step harness of the
reference (losses, clamping; utils.py:21-25,172-175)."""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib


def stream_handle(device: torch.device | None = None) -> int:
    """cudaStream_t of torch's current stream on `device` (0 = legacy default)."""
    if device is not None and device.type != "cuda":
        raise RuntimeError("librcv kernels need CUDA tensors")
    return torch.cuda.current_stream(device).cuda_stream


def require_cuda(*tensors: torch.Tensor) -> None:
    for t in tensors:
        if not isinstance(t, torch.Tensor) or not t.is_cuda:
            raise RuntimeError("librcv kernels need CUDA tensors")
        if t.dtype != torch.float32:
            raise TypeError("librcv kernels need float32 tensors")


class _LossOp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, img, ref, kind):
        img_c = img.detach().contiguous()
        ref_c = ref.detach().to(img.device, torch.float32).contiguous()
        require_cuda(img_c, ref_c)
        if img_c.shape != ref_c.shape:
            raise ValueError(f"image shape {tuple(img_c.shape)} != reference shape {tuple(ref_c.shape)}")
        lib = _lib.load()
        n = img_c.numel()
        ws = torch.empty(int(lib.rcv_loss_workspace_bytes(n)), dtype=torch.uint8, device=img_c.device)
        loss = torch.empty((), dtype=torch.float32, device=img_c.device)
        grad = torch.empty_like(img_c) if img.requires_grad else None
        _lib.check(
            lib.rcv_loss(
                kind, img_c.data_ptr(), ref_c.data_ptr(), n, loss.data_ptr(),
                grad.data_ptr() if grad is not None else None, ws.data_ptr(), stream_handle(img_c.device),
            ),
            "rcv_loss",
        )
        ctx.save_for_backward(grad if grad is not None else loss)
        ctx.has_grad = grad is not None
        return loss

    @staticmethod
    def backward(ctx, g):
        (grad,) = ctx.saved_tensors
        if not ctx.has_grad:
            return None, None, None
        return grad * g, None, None


def l2_loss(img: torch.Tensor, ref: torch.Tensor) -> torch.Tensor:
    """mean((img - ref)^2) with its gradient computed in the same kernel."""
    return _LossOp.apply(img, ref, _lib.LOSS_L2)


def l1_loss(img: torch.Tensor, ref: torch.Tensor) -> torch.Tensor:
    """mean(|img - ref|) with its gradient computed in the same kernel."""
    return _LossOp.apply(img, ref, _lib.LOSS_L1)


def clamp_(t: torch.Tensor, lo: float, hi: float) -> torch.Tensor:
    """In-place clamp of a float32 CUDA tensor."""
    require_cuda(t)
    if not t.is_contiguous():
        raise ValueError("clamp_ needs a contiguous tensor")
    _lib.check(
        _lib.load().rcv_clamp(t.data_ptr(), t.numel(), float(lo), float(hi), stream_handle(t.device)), "rcv_clamp"
    )
    return t


def clamp(params: dict, opt) -> None:
    """utils.clamp (utils.py:172-175): clamps every optimised variable that
    declares a 'clamp' range."""
    for key, param in params["variables"].items():
        if "clamp" in param:
            with torch.no_grad():
                clamp_(opt[key].data, param["clamp"][0], param["clamp"][1])


def upsample_grid(t: torch.Tensor, shape=None) -> torch.Tensor:
    """``dr.upsample`` of a tensor: nearest-neighbour up-sampling, every
    element repeated along each axis by the ratio of the target shape to the
    source shape (a whole multiple; Dr.Jit's documented behaviour for
    tensors).  Default target: twice the resolution of every axis but the
    last (the channels), as utils.upsample asks for (utils.py:181-183)."""
    if shape is None:
        shape = (*[2 * x for x in t.shape[:-1]], t.shape[-1])
    if len(shape) != t.dim():
        raise ValueError(f"upsample: target shape {tuple(shape)} does not match a {t.dim()}-D tensor")
    out = t
    for axis, (a, b) in enumerate(zip(t.shape, shape)):
        if b % a:
            raise ValueError(f"upsample: target extent {b} is not a multiple of {a} (axis {axis})")
        if b != a:
            out = out.repeat_interleave(b // a, dim=axis)
    return out


def upsample(scene, params: dict, opt, integrator) -> None:
    """utils.upsample (utils.py:177-192): doubles the resolution of every
    optimised grid (4-D) or texture (3-D) tensor in the optimiser, re-sizes
    the majorant supergrid of the density when ``use_majorant_supergrid`` is
    set (utils.adjust_majorant_res_factor, utils.py:27-43) and resets the
    integrator's control-variate state.  The next ``params.update(opt)``
    hands the new grids to the scene."""
    from . import scenes

    for key in params["variables"]:
        t = opt[key]
        if not isinstance(t, torch.Tensor):
            raise TypeError(f"Upsampling is only supported for tensors, got type {type(t)}.")
        if t.dim() not in (3, 4):
            raise ValueError(f"Upsampling expects a 3 or 4D tensor. Got {t.dim()}.")
        opt[key] = upsample_grid(t.detach())
        if ".sigma_t." in key and params.get("use_majorant_supergrid", False):
            new_res = tuple(opt[key].shape)
            for shape in scene.shapes():
                med = shape.interior_medium() if hasattr(shape, "interior_medium") else None
                if med is not None and hasattr(med, "set_majorant_resolution_factor"):
                    med.set_majorant_resolution_factor(scenes.majorant_factor_for(new_res[:3]))
    integrator.reset()


def upsample_steps(n_steps: int, fractions) -> list[int]:
    """Iterations at which run_opt upsamples (optimize.py:69-72)."""
    return [int(n_steps * w) for w in fractions]


def sample_tea_32(v0: int, v1: int) -> tuple[int, int]:
    return _lib.sample_tea_32(v0, v1)


def counters_tensor(device) -> torch.Tensor:
    return torch.zeros(_lib.COUNTER_COUNT, dtype=torch.int64, device=device)


def as_ptr(t: torch.Tensor | None):
    return None if t is None else C.c_void_p(t.data_ptr())
