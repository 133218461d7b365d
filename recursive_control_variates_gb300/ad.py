"""``Adam`` optimizer with the interface of ``mi.ad.Adam`` used by the
reference (optimize.py:90,127; utils.py:62-87,172-175): dictionary-style
variables, per-variable learning rates, and a GPU step (rcv_adam_step) that
applies the update, an optional clamp and resets the gradient.

Update rule (Kingma & Ba 2015, bias correction folded into the step size):
    m <- b1 m + (1-b1) g ;  v <- b2 v + (1-b2) g^2
    p <- p - lr sqrt(1-b2^t)/(1-b1^t) * m / (sqrt(v) + eps)
"""
from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .utils import require_cuda, stream_handle


class Adam:
    def __init__(self, lr: float, beta_1: float = 0.9, beta_2: float = 0.999, epsilon: float = 1e-8,
                 params: dict | None = None, device: str | torch.device = "cuda"):
        if not 0 <= beta_1 < 1 or not 0 <= beta_2 < 1:
            raise ValueError("Adam betas must be in [0, 1)")
        self.lr = float(lr)
        self.beta_1 = float(beta_1)
        self.beta_2 = float(beta_2)
        self.epsilon = float(epsilon)
        self.device = torch.device(device)
        self.variables: dict[str, torch.Tensor] = {}
        self.state: dict[str, list] = {}
        self.lr_per_key: dict[str, float] = {}
        self.bounds: dict[str, tuple[float, float]] = {}
        if params:
            for k, v in params.items():
                self[k] = v

    def keys(self):
        return self.variables.keys()

    def items(self):
        return self.variables.items()

    def __contains__(self, key):
        return key in self.variables

    def __getitem__(self, key) -> torch.Tensor:
        return self.variables[key]

    def __setitem__(self, key, value):
        if isinstance(value, torch.Tensor):
            t = value.detach().to(self.device, torch.float32)
        else:
            t = torch.as_tensor(np.asarray(value, np.float32), device=self.device)
        t = t.clone().contiguous().requires_grad_(True)
        old = self.variables.get(key)
        self.variables[key] = t
        if old is None or old.shape != t.shape:
            self.reset(key)

    def reset(self, key):
        t = self.variables[key]
        self.state[key] = [0, torch.zeros_like(t.detach()), torch.zeros_like(t.detach())]

    def set_learning_rate(self, lr):
        if isinstance(lr, dict):
            self.lr_per_key.update({k: float(v) for k, v in lr.items()})
        else:
            self.lr = float(lr)
            self.lr_per_key.clear()

    def set_bounds(self, key, lo: float, hi: float):
        """Clamp applied inside the step kernel (utils.clamp of the reference)."""
        self.bounds[key] = (float(lo), float(hi))

    def step(self):
        lib = _lib.load()
        for key, p in self.variables.items():
            g = p.grad
            if g is None:
                continue
            require_cuda(p)
            if not g.is_contiguous():
                g = g.contiguous()
                p.grad = g
            st = self.state[key]
            st[0] += 1
            lo, hi = self.bounds.get(key, (-np.inf, np.inf))
            lr = self.lr_per_key.get(key, self.lr)
            _lib.check(
                lib.rcv_adam_step(
                    p.data.data_ptr(), g.data_ptr(), st[1].data_ptr(), st[2].data_ptr(), p.numel(), st[0], lr,
                    self.beta_1, self.beta_2, self.epsilon, float(lo), float(hi), 1, stream_handle(p.device),
                ),
                "rcv_adam_step",
            )
