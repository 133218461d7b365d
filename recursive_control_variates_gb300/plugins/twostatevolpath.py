"""Two-state volumetric path-replay integrator (``twostateprbvolpath``) and
its single-state counterpart (``prbvolpath``).

Interface of plugins/twostatevolpath.py:11-138 of the reference:
``render_twostates(scene, sensor, seed, spp) -> (H, F)`` renders the previous
and current medium parameters with shared random numbers; ``render`` renders
the current parameters only; ``render_backward`` back-propagates an image
gradient into the current parameters by path replay.  All three run on the
GPU through librcv.
"""
from __future__ import annotations

import ctypes as C

import torch

from .. import _lib, profiling
from ..core import CubeShape, HeterogeneousMedium, Properties, TwoStateMedium
from ..utils import stream_handle

# linear sRGB -> CIE XYZ (D65), for the `xyz` option
_SRGB_TO_XYZ = torch.tensor(
    [[0.412453, 0.357580, 0.180423], [0.212671, 0.715160, 0.072169], [0.019334, 0.119193, 0.950227]],
    dtype=torch.float32,
)


class _VolumeIntegratorBase:
    two_state = False

    def __init__(self, props: Properties):
        self.max_depth = int(props.get("max_depth", 6))
        self.rr_depth = int(props.get("rr_depth", 5))
        self.hide_emitters = bool(props.get("hide_emitters", False))
        self.xyz = bool(props.get("xyz", False))
        # scheduling knobs of the persistent tracer (results do not depend on them)
        self.batch = int(props.get("batch", 0))
        self.blocks_per_sm = int(props.get("blocks_per_sm", 0))
        self.defer = int(props.get("defer", 0))
        order = props.get("order", "cost")
        if order not in _lib.ORDERS:
            raise ValueError(f"unknown pixel order {order!r}")
        self.order = _lib.ORDERS[order]
        if self.max_depth < -1:
            raise ValueError("max_depth must be -1 (infinite) or non-negative")
        # run the adjoint's radiance pass beside the primal render (rcv.render)
        self.overlap_adjoint = bool(props.get("overlap_adjoint", True))
        # ... in the same persistent launch as a two-state render
        # (rcv_render_twostates_volume_and_adjoint_radiance) rather than on a
        # side stream
        self.pair_adjoint = bool(props.get("pair_adjoint", True))
        # gradient from an event tape of the radiance pass ("tape") or from
        # replayed path segments ("replay"); the same gradient either way
        adjoint = props.get("adjoint", "tape")
        if adjoint not in _lib.ADJOINTS:
            raise ValueError(f"unknown adjoint {adjoint!r}")
        self.adjoint = _lib.ADJOINTS[adjoint]
        self.tape_events_per_path = int(props.get("tape_events_per_path", 0))
        if not 0 <= self.tape_events_per_path <= 16:
            raise ValueError("tape_events_per_path must be in [0, 16]")
        # accumulate the RCV_COUNTER_* event counts into counters() (the
        # counting tracer variants hold the counts in registers)
        self.count_events = bool(props.get("count_events", False))
        self.is_checked = False
        self._counters: dict[torch.device, torch.Tensor] = {}
        self._scratch: dict[torch.device, torch.Tensor] = {}
        self._adj_scratch: dict[torch.device, torch.Tensor] = {}
        self._side: dict[torch.device, torch.cuda.Stream] = {}
        self._ticket = None  # (key, done event) of an adjoint radiance pass started ahead
        self._pending = None  # a prepared radiance pass the next two-state render may run with it
        self.last_primal_call = None

    # ------------------------------------------------------------- helpers
    def options(self, scene=None) -> _lib.VolpathOptions:
        """Tracer options; with a scene, also its environment map (None for
        the constant environment)."""
        o = _lib.VolpathOptions()
        o.max_depth = self.max_depth
        o.rr_depth = self.rr_depth
        o.hide_emitters = int(self.hide_emitters)
        o.batch = self.batch
        o.blocks_per_sm = self.blocks_per_sm
        o.defer = self.defer
        o.order = self.order
        o.adjoint = self.adjoint
        o.tape_events_per_path = self.tape_events_per_path
        o.separate_tracers = 0 if self.pair_adjoint else 1
        env = scene.envmap() if scene is not None and hasattr(scene, "envmap") else None
        o.envmap = C.addressof(env.c_struct()) if env is not None else None
        return o

    def counters_ptr(self, device):
        """Device address of counters() when counting, else None."""
        return self.counters(device).data_ptr() if self.count_events else None

    def counters(self, device) -> torch.Tensor:
        device = torch.device(device)
        if device not in self._counters:
            self._counters[device] = torch.zeros(_lib.COUNTER_COUNT, dtype=torch.int64, device=device)
        return self._counters[device]

    def scratch(self, device, sensor, spp: int, mode: int) -> int:
        """256-B aligned device address of the tracer scratch (grown on
        demand; reused by later calls, which are ordered on the stream)."""
        device = torch.device(device)
        f = sensor.film()
        need = int(_lib.load().rcv_render_workspace_bytes(f.width, f.height, spp, mode)) + 256
        buf = self._scratch.get(device)
        if buf is None or buf.numel() < need:
            # zeroed once: the per-pixel cost it carries starts at zero
            buf = torch.zeros(need, dtype=torch.uint8, device=device)
            self._scratch[device] = buf
        return (buf.data_ptr() + 255) & ~255

    def adjoint_scratch(self, device, sensor, spp: int) -> int:
        """256-B aligned scratch of the adjoint launches (its own buffer, so
        an adjoint radiance pass on the side stream never shares scratch with
        a primal render)."""
        device = torch.device(device)
        f = sensor.film()
        need = int(_lib.load().rcv_render_workspace_bytes(f.width, f.height, spp, _lib.MODE_ADJOINT)) + 256
        buf = self._adj_scratch.get(device)
        if buf is None or buf.numel() < need:
            self._drain_ticket(device)  # the old buffer may still be in use
            buf = torch.zeros(need, dtype=torch.uint8, device=device)
            self._adj_scratch[device] = buf
        return (buf.data_ptr() + 255) & ~255

    def _drain_ticket(self, device):
        t, self._ticket = self._ticket, None
        if t is not None:
            torch.cuda.current_stream(device).wait_event(t[1])

    def _adjoint_key(self, scene, medium, sensor, seed: int, spp: int):
        o = self.options(scene)
        return (id(medium), medium.version, id(sensor), seed & 0xFFFFFFFF, int(spp),
                tuple(getattr(o, f) for f, _ in o._fields_))

    def prefetch_adjoint(self, scene, sensor=0, seed: int = 0, spp: int = 0):
        """Prepares the adjoint's first launch (each path's radiance and its
        scatter checkpoints), which does not depend on the image gradient.
        Returns a function that enqueues it on a side stream, ordered after
        the medium's packing but not after the work enqueued in between (the
        primal render), or None when there is nothing to overlap.  With
        ``pair_adjoint`` (the default) a ``render_twostates`` of the same
        medium state, sensor and options called before that function runs
        the pass in its own launch instead, and the function does nothing.
        ``render_backward`` with the same arguments then only replays."""
        if not self.overlap_adjoint:
            return None
        medium = self._checked_medium(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        dev = medium.device
        main = torch.cuda.current_stream(dev)
        m = medium.prepare(main.cuda_stream)
        s = sensor.c_struct()
        o = self.options(scene)
        ws = self.adjoint_scratch(dev, sensor, spp)
        packed = torch.cuda.Event()
        packed.record(main)
        key = self._adjoint_key(scene, medium, sensor, seed, spp)
        side = self._side.get(dev)
        if side is None:
            side = self._side[dev] = torch.cuda.Stream(dev)
        counters = self.counters_ptr(dev)
        pending = {"key": key, "seed": seed, "spp": spp, "ws": ws, "used": False}
        self._pending = pending if self.pair_adjoint else None

        def launch():
            if self._pending is pending:
                self._pending = None
            if pending["used"]:
                return  # it ran in the launch of the two-state render
            self._drain_ticket(dev)
            side.wait_event(packed)
            with torch.cuda.stream(side), profiling.region("trace_adjoint_radiance", dev):
                _lib.check(
                    _lib.load().rcv_render_adjoint_radiance(
                        C.byref(m), C.byref(s), C.byref(o), seed & 0xFFFFFFFF, spp, ws, counters,
                        side.cuda_stream,
                    ),
                    "rcv_render_adjoint_radiance",
                )
            done = torch.cuda.Event()
            done.record(side)
            medium.add_reader(done)
            self._ticket = (key, done)

        return launch

    @staticmethod
    def medium_of(scene):
        for shape in scene.shapes():
            if isinstance(shape, CubeShape):
                m = shape.interior_medium()
                if m is not None:
                    return m
        return None

    @staticmethod
    def sensor_of(scene, sensor):
        if isinstance(sensor, int):
            if len(scene.sensors()) == 0:
                raise Exception("No sensor specified! Add a sensor in the scene description.")
            return scene.sensors()[sensor]
        return sensor

    @staticmethod
    def resolve_spp(sensor, spp: int) -> int:
        return int(spp) if spp and spp > 0 else int(sensor.sampler().sample_count)

    def _post(self, img: torch.Tensor) -> torch.Tensor:
        if not self.xyz:
            return img
        m = _SRGB_TO_XYZ.to(img.device)
        return img @ m.T

    def _image(self, sensor, device) -> torch.Tensor:
        f = sensor.film()
        return torch.empty((f.height, f.width, 3), dtype=torch.float32, device=device)

    # --------------------------------------------------------------- render
    def render(self, scene, sensor=0, seed: int = 0, spp: int = 0, develop: bool = True, evaluate: bool = True):
        """Single-state render of the current parameters."""
        medium = self._checked_medium(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        st = stream_handle(medium.device)
        m = medium.prepare(st)
        s = sensor.c_struct()
        o = self.options(scene)
        img = self._image(sensor, medium.device)
        with profiling.region("trace_single", medium.device):
            _lib.check(
                _lib.load().rcv_render_volume(
                    C.byref(m), C.byref(s), C.byref(o), seed & 0xFFFFFFFF, spp, img.data_ptr(),
                    self.scratch(medium.device, sensor, spp, _lib.MODE_SINGLE),
                    self.counters_ptr(medium.device), st,
                ),
                "rcv_render_volume",
            )
        return self._post(img)

    def render_backward(self, scene, params, grad_in: torch.Tensor, sensor=0, seed: int = 0, spp: int = 0):
        """Path-replay adjoint on the current parameters.

        Returns ``{key: gradient}`` for the differentiable medium parameters
        present in ``params`` (density ``...sigma_t.data`` and, when the
        medium has an albedo grid, ``...albedo.data``)."""
        medium = self._checked_medium(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        if self.xyz:
            grad_in = grad_in @ _SRGB_TO_XYZ.to(grad_in.device)
        g = grad_in.detach().to(medium.device, torch.float32).contiguous()
        f = sensor.film()
        if tuple(g.shape) != (f.height, f.width, 3):
            raise ValueError(f"grad_in has shape {tuple(g.shape)}, expected {(f.height, f.width, 3)}")
        dev = medium.device
        ticket, key = self._ticket, None
        if ticket is not None:
            key = self._adjoint_key(scene, medium, sensor, seed, spp)
        self._drain_ticket(dev)  # orders this stream after a radiance pass started ahead
        st = stream_handle(dev)
        m = medium.prepare(st)
        s = sensor.c_struct()
        o = self.options(scene)
        dx, dy, dz = medium.dims
        gd = torch.zeros((dz, dy, dx, 1), dtype=torch.float32, device=dev)
        ga = medium.albedo_grad_buffer()
        ws = self.adjoint_scratch(dev, sensor, spp)
        # the radiance pass already ran for exactly these arguments: replay only
        fn = ("rcv_render_backward_replay" if ticket is not None and ticket[0] == key and medium.version == key[1]
              else "rcv_render_backward_volume")
        self.last_adjoint_call = fn
        with profiling.region("trace_adjoint", dev):
            _lib.check(
                getattr(_lib.load(), fn)(
                    C.byref(m), C.byref(s), C.byref(o), seed & 0xFFFFFFFF, spp, g.data_ptr(), gd.data_ptr(),
                    ga.data_ptr() if ga is not None else None, ws, self.counters_ptr(dev), st,
                ),
                fn,
            )
        out = {}
        keys = list(params.keys()) if params is not None else []
        for key in keys:
            owner, sub = params.owner_of(key)
            if owner is not medium:
                continue
            if sub == "sigma_t.data":
                out[key] = gd
            elif sub == "albedo.data" and ga is not None:
                out[key] = ga
        return out

    def render_forward(self, scene, params, sensor=0, seed: int = 0, spp: int = 0, tangents=None):
        """Forward-mode derivative of the render of the current parameters:
        the (H, W, 3) image derivative along the tangent of each
        differentiable medium parameter (density ``...sigma_t.data``,
        albedo grid ``...albedo.data``).  ``tangents`` maps keys to tensors
        shaped like the parameters; by default each parameter tensor's
        ``.grad`` is its tangent (the role of ``dr.grad`` in the reference's
        forward mode).  Estimated by path replay from ``seed`` with ``spp``
        paths per pixel (rcv_render_forward_volume)."""
        medium = self._checked_medium(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        dev = medium.device
        td = ta = None
        keys = list(params.keys()) if params is not None else []
        for key in keys:
            owner, sub = params.owner_of(key)
            if owner is not medium:
                continue
            if tangents is not None:
                t = tangents.get(key)
            else:
                v = params[key]
                t = v.grad if isinstance(v, torch.Tensor) else None
            if t is None:
                continue
            t = t.detach().to(dev, torch.float32).contiguous()
            if sub == "sigma_t.data":
                dx, dy, dz = medium.dims
                td = t.reshape(dz, dy, dx)
            elif sub == "albedo.data" and medium.has_albedo_grid:
                ax, ay, az = medium.albedo_dims
                ta = t.reshape(az, ay, ax, 3)
        f = sensor.film()
        out = torch.zeros((f.height, f.width, 3), dtype=torch.float32, device=dev)
        if td is None and ta is None:
            return self._post(out)
        self._drain_ticket(dev)  # the call overwrites the adjoint scratch and the gradient records
        st = stream_handle(dev)
        m = medium.prepare(st)
        s = sensor.c_struct()
        o = self.options(scene)
        with profiling.region("trace_forward", dev):
            _lib.check(
                _lib.load().rcv_render_forward_volume(
                    C.byref(m), C.byref(s), C.byref(o), seed & 0xFFFFFFFF, spp,
                    td.data_ptr() if td is not None else None, ta.data_ptr() if ta is not None else None,
                    out.data_ptr(), self.adjoint_scratch(dev, sensor, spp), self.counters_ptr(dev), st,
                ),
                "rcv_render_forward_volume",
            )
        return self._post(out)

    def _checked_medium(self, scene):
        raise NotImplementedError


class TwoStatePRBVolpathIntegrator(_VolumeIntegratorBase):
    """``twostateprbvolpath`` (plugins/twostatevolpath.py:11-482)."""

    two_state = True

    def check_scene(self, scene):
        # plugins/twostatevolpath.py:67-78
        if self.is_checked:
            return
        self.is_checked = True
        if not isinstance(self.medium_of(scene), TwoStateMedium):
            self.is_checked = False
            raise RuntimeError("No TwoStateMedium found in the scene!")

    def _checked_medium(self, scene):
        self.check_scene(scene)
        return self.medium_of(scene)

    def render_twostates(self, scene, sensor=0, seed: int = 0, spp: int = 1):
        """Returns (H, F): images of the previous and current parameters
        rendered with the same random numbers (plugins/twostatevolpath.py:91-138)."""
        medium = self._checked_medium(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        st = stream_handle(medium.device)
        m = medium.prepare(st)
        s = sensor.c_struct()
        o = self.options(scene)
        H = self._image(sensor, medium.device)
        F = self._image(sensor, medium.device)
        ws = self.scratch(medium.device, sensor, spp, _lib.MODE_TWOSTATE)
        # an adjoint radiance pass prepared for this medium state, sensor and
        # options runs in the same launch
        pend, self._pending = self._pending, None
        key = self._adjoint_key(scene, medium, sensor, 0, 0)
        if pend is not None and (pend["key"][:3] != key[:3] or pend["key"][5:] != key[5:]):
            pend = None
        with profiling.region("trace_twostate", medium.device):
            if pend is None:
                fn = "rcv_render_twostates_volume"
                rc = _lib.load().rcv_render_twostates_volume(
                    C.byref(m), C.byref(s), C.byref(o), seed & 0xFFFFFFFF, spp, H.data_ptr(), F.data_ptr(), ws,
                    self.counters_ptr(medium.device), st,
                )
            else:
                fn = "rcv_render_twostates_volume_and_adjoint_radiance"
                self._drain_ticket(medium.device)  # the call overwrites the adjoint scratch
                rc = _lib.load().rcv_render_twostates_volume_and_adjoint_radiance(
                    C.byref(m), C.byref(s), C.byref(o), seed & 0xFFFFFFFF, spp, H.data_ptr(), F.data_ptr(), ws,
                    pend["seed"] & 0xFFFFFFFF, pend["spp"], pend["ws"], self.counters_ptr(medium.device), st,
                )
            _lib.check(rc, fn)
        self.last_primal_call = fn
        if pend is not None:
            done = torch.cuda.Event()
            done.record(torch.cuda.current_stream(medium.device))
            medium.add_reader(done)
            self._ticket = (pend["key"], done)
            pend["used"] = True
        self.primal_image_old, self.primal_image_new = self._post(H), self._post(F)
        return self.primal_image_old, self.primal_image_new

    def to_string(self):
        return f"TwoStatePRBVolpathIntegrator[max_depth = {self.max_depth}]"


class PRBVolpathIntegrator(_VolumeIntegratorBase):
    """Single-state volumetric path replay (``prbvolpath``): the integrator the
    reference pairs with the baseline method (experiments.py:131).  Accepts a
    plain heterogeneous medium or a two-state one (then renders ``new``)."""

    def _checked_medium(self, scene):
        m = self.medium_of(scene)
        if not isinstance(m, (HeterogeneousMedium, TwoStateMedium)):
            raise RuntimeError("No heterogeneous medium found in the scene!")
        return m

    def to_string(self):
        return f"PRBVolpathIntegrator[max_depth = {self.max_depth}]"
