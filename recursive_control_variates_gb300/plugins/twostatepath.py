"""Surface two-state path-replay integrator (``twostateprb``,
plugins/twostatepath.py:97-364 of the reference), on the GPU through librcv.

``render_twostates(scene, sensor, seed, spp) -> (H, F)`` renders the previous
and current BSDF states with shared random numbers; ``render`` renders the
current state; ``render_backward`` back-propagates an image gradient into the
ground texture (``<plane>.bsdf.reflectance.data``) by path replay.
"""
from __future__ import annotations

import ctypes as C

import torch

from .. import _lib, profiling
from ..core import Properties
from ..surface import SurfaceSceneView, TwoStateBSDF
from ..utils import stream_handle


class TwoStatePRBIntegrator:
    """``twostateprb``: surface form of the two-state tracer."""

    two_state = True

    def __init__(self, props: Properties):
        self.max_depth = int(props.get("max_depth", 6))
        self.rr_depth = int(props.get("rr_depth", 5))
        self.hide_emitters = bool(props.get("hide_emitters", False))
        self.xyz = bool(props.get("xyz", False))
        if self.xyz:
            raise ValueError("xyz output is not supported by the surface tracer")
        if self.max_depth < -1:
            raise ValueError("max_depth must be -1 (infinite) or non-negative")
        self.batch = int(props.get("batch", 0))
        self.blocks_per_sm = int(props.get("blocks_per_sm", 0))
        # adjoint: texture vertices recorded on a tape ("tape") or the paths
        # traced a second time ("replay"); the same gradient either way
        adjoint = props.get("adjoint", "tape")
        if adjoint not in _lib.ADJOINTS:
            raise ValueError(f"unknown adjoint {adjoint!r}")
        self.adjoint = _lib.ADJOINTS[adjoint]
        self.tape_events_per_path = int(props.get("tape_events_per_path", 0))
        if not 0 <= self.tape_events_per_path <= 16:
            raise ValueError("tape_events_per_path must be in [0, 16]")
        self.is_checked = False
        self._counters: dict[torch.device, torch.Tensor] = {}
        self._scratch: dict[torch.device, torch.Tensor] = {}

    # ------------------------------------------------------------- helpers
    def options(self) -> _lib.VolpathOptions:
        o = _lib.VolpathOptions()
        o.max_depth, o.rr_depth, o.hide_emitters = self.max_depth, self.rr_depth, int(self.hide_emitters)
        o.batch, o.blocks_per_sm = self.batch, self.blocks_per_sm
        o.order = _lib.ORDER_ROW_MAJOR
        o.adjoint, o.tape_events_per_path = self.adjoint, self.tape_events_per_path
        return o

    def counters(self, device) -> torch.Tensor:
        device = torch.device(device)
        if device not in self._counters:
            self._counters[device] = torch.zeros(_lib.COUNTER_COUNT, dtype=torch.int64, device=device)
        return self._counters[device]

    def scratch(self, device, sensor, spp: int, mode: int) -> int:
        device = torch.device(device)
        f = sensor.film()
        need = int(_lib.load().rcv_render_workspace_bytes(f.width, f.height, spp, mode)) + 256
        buf = self._scratch.get(device)
        if buf is None or buf.numel() < need:
            buf = torch.empty(need, dtype=torch.uint8, device=device)
            self._scratch[device] = buf
        return (buf.data_ptr() + 255) & ~255

    def check_scene(self, scene):
        # plugins/twostatepath.py:152-166
        if self.is_checked:
            return
        has_twostate = False
        for shape in scene.shapes():
            if isinstance(getattr(shape, "bsdf", None), TwoStateBSDF):
                has_twostate = True
            med = shape.interior_medium() if hasattr(shape, "interior_medium") else None
            if med is not None and type(med).__name__ == "TwoStateMedium":
                raise ValueError("TwoStateMedium is not supported in two state prb integrator!")
        if not has_twostate:
            raise RuntimeError("No TwoStateBSDF found in the scene!")
        self.is_checked = True

    def view(self, scene) -> SurfaceSceneView:
        self.check_scene(scene)
        v = getattr(scene, "_surface_view", None)
        if v is None:
            v = SurfaceSceneView(scene)
            scene._surface_view = v
        return v

    @staticmethod
    def sensor_of(scene, sensor):
        return scene.sensors()[sensor] if isinstance(sensor, int) else sensor

    @staticmethod
    def resolve_spp(sensor, spp):
        return int(spp) if spp and spp > 0 else int(sensor.sampler().sample_count)

    def _image(self, sensor, device):
        f = sensor.film()
        return torch.empty((f.height, f.width, 3), dtype=torch.float32, device=device)

    # ------------------------------------------------------------- renders
    def render_twostates(self, scene, sensor=0, seed: int = 0, spp: int = 1):
        v = self.view(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        st = stream_handle(v.device)
        s = v.prepare(st)
        cam, o = sensor.c_struct(), self.options()
        H, F = self._image(sensor, v.device), self._image(sensor, v.device)
        with profiling.region("trace_surface_twostate", v.device):
            _lib.check(
                _lib.load().rcv_render_twostates_surface(
                    C.byref(s), C.byref(cam), C.byref(o), seed & 0xFFFFFFFF, spp, H.data_ptr(), F.data_ptr(),
                    self.scratch(v.device, sensor, spp, _lib.MODE_TWOSTATE), self.counters(v.device).data_ptr(), st,
                ),
                "rcv_render_twostates_surface",
            )
        self.primal_image_old, self.primal_image_new = H, F
        return H, F

    def render(self, scene, sensor=0, seed: int = 0, spp: int = 0, develop: bool = True, evaluate: bool = True):
        v = self.view(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        st = stream_handle(v.device)
        s = v.prepare(st)
        cam, o = sensor.c_struct(), self.options()
        img = self._image(sensor, v.device)
        with profiling.region("trace_surface_single", v.device):
            _lib.check(
                _lib.load().rcv_render_surface(
                    C.byref(s), C.byref(cam), C.byref(o), seed & 0xFFFFFFFF, spp, img.data_ptr(),
                    self.scratch(v.device, sensor, spp, _lib.MODE_SINGLE), self.counters(v.device).data_ptr(), st,
                ),
                "rcv_render_surface",
            )
        return img

    def render_backward(self, scene, params, grad_in, sensor=0, seed: int = 0, spp: int = 0):
        v = self.view(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        g = grad_in.detach().to(v.device, torch.float32).contiguous()
        f = sensor.film()
        if tuple(g.shape) != (f.height, f.width, 3):
            raise ValueError(f"grad_in has shape {tuple(g.shape)}, expected {(f.height, f.width, 3)}")
        st = stream_handle(v.device)
        s = v.prepare(st)
        cam, o = sensor.c_struct(), self.options()
        gt = torch.zeros_like(v.bsdf.new.texture.data)
        with profiling.region("trace_surface_adjoint", v.device):
            _lib.check(
                _lib.load().rcv_render_backward_surface(
                    C.byref(s), C.byref(cam), C.byref(o), seed & 0xFFFFFFFF, spp, g.data_ptr(), gt.data_ptr(),
                    self.scratch(v.device, sensor, spp, _lib.MODE_ADJOINT), self.counters(v.device).data_ptr(), st,
                ),
                "rcv_render_backward_surface",
            )
        out = {}
        for key in (params.keys() if params is not None else []):
            owner, sub = params.owner_of(key)
            if owner is v.bsdf and sub == "reflectance.data":
                out[key] = gt
        return out

    def render_forward(self, scene, params, sensor=0, seed: int = 0, spp: int = 0, tangents=None):
        """Forward-mode derivative of the render of the current texture: the
        (H, W, 3) image derivative along the tangent of the textured BSDF's
        ``reflectance.data`` (``tangents[key]``, by default the parameter
        tensor's ``.grad``), by path replay (rcv_render_forward_surface)."""
        v = self.view(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        f = sensor.film()
        out = torch.zeros((f.height, f.width, 3), dtype=torch.float32, device=v.device)
        tex = None
        for key in (params.keys() if params is not None else []):
            owner, sub = params.owner_of(key)
            if owner is v.bsdf and sub == "reflectance.data":
                if tangents is not None:
                    tex = tangents.get(key)
                else:
                    p = params[key]
                    tex = p.grad if isinstance(p, torch.Tensor) else None
        if tex is None:
            return out
        t = tex.detach().to(v.device, torch.float32).contiguous().reshape(v.bsdf.new.texture.data.shape)
        st = stream_handle(v.device)
        s = v.prepare(st)
        cam, o = sensor.c_struct(), self.options()
        with profiling.region("trace_surface_forward", v.device):
            _lib.check(
                _lib.load().rcv_render_forward_surface(
                    C.byref(s), C.byref(cam), C.byref(o), seed & 0xFFFFFFFF, spp, t.data_ptr(), out.data_ptr(),
                    self.scratch(v.device, sensor, spp, _lib.MODE_ADJOINT), self.counters(v.device).data_ptr(), st,
                ),
                "rcv_render_forward_surface",
            )
        return out

    def to_string(self):
        return f"TwoStatePRBIntegrator[max_depth = {self.max_depth}]"
