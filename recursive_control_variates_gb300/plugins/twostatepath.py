"""Surface two-state path-replay integrator (``twostateprb``,
plugins/twostatepath.py:97-364 of the reference)."""
from __future__ import annotations

from ..core import Properties


class TwoStatePRBIntegrator:
    """``twostateprb``: surface form of the two-state tracer."""

    two_state = True

    def __init__(self, props: Properties):
        self.max_depth = int(props.get("max_depth", 6))
        self.rr_depth = int(props.get("rr_depth", 5))
        self.xyz = bool(props.get("xyz", False))
        self.is_checked = False

    def _unavailable(self, *a, **k):
        raise NotImplementedError("the surface two-state tracer is not built yet")

    render = render_twostates = render_backward = render_forward = _unavailable
