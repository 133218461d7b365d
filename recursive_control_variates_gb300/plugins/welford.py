"""EMA-Welford estimators on the device (plugins/welford.py of the reference).

``StatisticsEstimator`` keeps per-element exponential-moving-average mean,
variance and covariance of two images (H and F of the control variate);
``WelfordVarianceEstimator`` is the single-variable version.  Both hold a
scalar sample count ``n`` on the host (the reference keeps it as an opaque
scalar tensor, plugins/welford.py:17-18,43-44) and float32 ``beta1``/``beta2``.
"""
from __future__ import annotations

import ctypes as C

import torch

from .. import _lib
from ..utils import stream_handle


def _zeros_like(t: torch.Tensor) -> torch.Tensor:
    return torch.zeros_like(t, dtype=torch.float32)


class StatisticsEstimator:
    """plugins/welford.py:38-78"""

    def __init__(self, beta1: float = 0.9, beta2: float = 0.999):
        self.n = 0
        self.beta1 = float(beta1)
        self.beta2 = float(beta2)
        self.mean_x = self.mean_y = self.var_x = self.var_y = self.cov = None

    def _ensure(self, like: torch.Tensor) -> None:
        if self.mean_x is None or self.mean_x.shape != like.shape:
            self.mean_x, self.mean_y, self.var_x, self.var_y, self.cov = (_zeros_like(like) for _ in range(5))

    def state_struct(self, img, w_s, v_n) -> _lib.CvState:
        s = _lib.CvState()
        s.img, s.w_s, s.v_n = img.data_ptr(), w_s.data_ptr(), v_n.data_ptr()
        s.mean_x, s.mean_y = self.mean_x.data_ptr(), self.mean_y.data_ptr()
        s.var_x, s.var_y, s.cov = self.var_x.data_ptr(), self.var_y.data_ptr(), self.cov.data_ptr()
        return s

    def update(self, x: torch.Tensor, y: torch.Tensor) -> None:
        x = x.contiguous()
        y = y.contiguous()
        self._ensure(x)
        s = self.state_struct(self.mean_x, self.mean_x, self.mean_x)  # img/w_s/v_n unused
        cnt = C.c_int32(self.n)
        _lib.check(
            _lib.load().rcv_statistics_update(
                C.byref(s), x.numel(), x.data_ptr(), y.data_ptr(), C.byref(cnt), self.beta1, self.beta2,
                stream_handle(x.device),
            ),
            "StatisticsEstimator.update",
        )
        self.n = cnt.value

    def get(self):
        if self.mean_x is None:
            raise RuntimeError("StatisticsEstimator.get before any update")
        s = self.state_struct(self.mean_x, self.mean_x, self.mean_x)
        vx, vy, cv = torch.empty_like(self.var_x), torch.empty_like(self.var_y), torch.empty_like(self.cov)
        _lib.check(
            _lib.load().rcv_statistics_get(
                C.byref(s), vx.numel(), self.n, self.beta2, vx.data_ptr(), vy.data_ptr(), cv.data_ptr(),
                stream_handle(vx.device),
            ),
            "StatisticsEstimator.get",
        )
        return vx, vy, cv


class WelfordVarianceEstimator:
    """plugins/welford.py:4-36"""

    def __init__(self, beta1: float = 0.9, beta2: float = 0.999):
        self.n = 0
        self.beta1 = float(beta1)
        self.beta2 = float(beta2)
        self.mean = None
        self.var = None

    def update(self, x: torch.Tensor) -> None:
        x = x.contiguous()
        if self.mean is None or self.mean.shape != x.shape:
            self.mean, self.var = _zeros_like(x), _zeros_like(x)
        cnt = C.c_int32(self.n)
        _lib.check(
            _lib.load().rcv_welford_update(
                self.mean.data_ptr(), self.var.data_ptr(), x.numel(), x.data_ptr(), C.byref(cnt), self.beta1,
                self.beta2, stream_handle(x.device),
            ),
            "WelfordVarianceEstimator.update",
        )
        self.n = cnt.value

    def get(self) -> torch.Tensor:
        if self.var is None:
            raise RuntimeError("WelfordVarianceEstimator.get before any update")
        out = torch.empty_like(self.var)
        _lib.check(
            _lib.load().rcv_welford_get(
                self.var.data_ptr(), out.numel(), self.n, self.beta2, out.data_ptr(), stream_handle(out.device)
            ),
            "WelfordVarianceEstimator.get",
        )
        return out
