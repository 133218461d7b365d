"""Optional CUDA-event timing of librcv launches.

When a ``KernelTimer`` is active (``with KernelTimer() as t:``), the
integrators bracket each tracer launch with events recorded on the stream the
kernel is launched on, keyed by kernel name; ``t.summary()`` returns
per-kernel launch counts and mean durations.  Inactive, it costs one
attribute lookup per launch.
"""
from __future__ import annotations

import contextlib
from collections import defaultdict

import torch

_active: "KernelTimer | None" = None


class KernelTimer:
    def __init__(self):
        self.events = defaultdict(list)

    def __enter__(self):
        global _active
        self._prev = _active
        _active = self
        return self

    def __exit__(self, *exc):
        global _active
        _active = self._prev
        return False

    def summary(self) -> dict:
        torch.cuda.synchronize()
        out = {}
        for name, pairs in self.events.items():
            ms = [a.elapsed_time(b) for a, b in pairs]
            out[name] = {"launches": len(ms), "mean_ms": sum(ms) / len(ms), "total_ms": sum(ms)}
        return out


@contextlib.contextmanager
def region(name: str, device=None):
    t = _active
    if t is None:
        yield
        return
    s = torch.cuda.current_stream(device)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(s)
    try:
        yield
    finally:
        b.record(s)
        t.events[name].append((a, b))
