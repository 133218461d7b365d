"""Surface scene plugins: ground rectangle, spheres, rectangular area light,
diffuse / bitmap / two-state BSDFs.

The surface form of the reference (``twostateprb`` with the ``twostate`` BSDF,
plugins/twostatepath.py and plugins/twostatebsdf.py) is supported for this
scene family: a ground rectangle y = 0 (``rectangle`` with ``ground: true``,
half size ``half_size``) whose ``twostate`` diffuse BSDF holds an RGB bitmap,
diffuse ``sphere`` shapes, and one ``rectangle`` carrying an ``area``
emitter, parallel to the ground and facing down.  The optimised parameter key
is ``<plane name>.bsdf.reflectance.data`` (bitmap texture data, (H, W, 3)).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .core import Properties, _device, register_bsdf, register_object


class BitmapTexture:
    """``bitmap`` texture with in-memory ``data`` (H, W, 3): bilinear, repeat."""

    def __init__(self, props: Properties):
        if "filename" in props:
            raise ValueError("bitmap from files is not supported; pass 'data'")
        self.device = _device(props)
        t = props["data"]
        t = torch.as_tensor(np.asarray(t) if not isinstance(t, torch.Tensor) else t)
        t = t.detach().to(self.device, torch.float32).clone().contiguous()
        if t.dim() != 3 or t.shape[-1] != 3:
            raise ValueError(f"bitmap data must have shape (H, W, 3), got {tuple(t.shape)}")
        self.data = t


class DiffuseBSDF:
    def __init__(self, props: Properties):
        refl = props.get("reflectance", 0.5)
        self.texture = None
        self.value = (0.5, 0.5, 0.5)
        if isinstance(refl, BitmapTexture):
            self.texture = refl
        else:
            if isinstance(refl, dict):
                refl = refl.get("value", 0.5)
            a = np.broadcast_to(np.asarray(refl, np.float64), (3,))
            self.value = tuple(float(np.float32(v)) for v in a)


class TwoStateBSDF:
    """``twostate`` BSDF (plugins/twostatebsdf.py:4-81): sampling, pdf and eval
    use ``new``, eval_old uses ``old``; traverse exposes ``incoming``;
    parameters_changed rotates old <- new <- incoming."""

    def __init__(self, props: Properties):
        self.old, self.new, self.incoming = props["old"], props["new"], props["incoming"]
        for b in (self.old, self.new, self.incoming):
            if not isinstance(b, DiffuseBSDF):
                raise ValueError("twostate BSDF expects diffuse BSDFs for old/new/incoming")
        kinds = {b.texture is None for b in (self.old, self.new, self.incoming)}
        if len(kinds) != 1:
            raise ValueError("old/new/incoming must all be textured or all be constant")
        self.textured = self.new.texture is not None
        if self.textured and not (self.old.texture.data.shape == self.new.texture.data.shape
                                  == self.incoming.texture.data.shape):
            raise ValueError("old/new/incoming textures must have the same resolution")
        self._dirty = True

    def traverse(self) -> dict[str, torch.Tensor]:
        if self.textured:
            return {"reflectance.data": self.incoming.texture.data}
        return {}

    def parameters_changed(self, keys=None) -> None:
        o, n, i = self.old, self.new, self.incoming
        if self.textured:
            o.texture.data, n.texture.data = n.texture.data, o.texture.data
            n.texture.data.copy_(i.texture.data)
        o.value, n.value = n.value, i.value
        self._dirty = True


class AreaEmitter:
    def __init__(self, props: Properties):
        rad = props.get("radiance", 1.0)
        if isinstance(rad, dict):
            rad = rad.get("value", 1.0)
        self.radiance = tuple(float(np.float32(v)) for v in np.broadcast_to(np.asarray(rad, np.float64), (3,)))


class RectangleShape:
    """Axis-aligned rectangle parallel to y = 0: the ground (``ground: true``,
    centred at the origin, reflective) or an area light (``emitter``)."""

    is_surface_shape = True

    def __init__(self, props: Properties):
        self.ground = bool(props.get("ground", False))
        hs = np.broadcast_to(np.asarray(props.get("half_size", 1.0), np.float64), (2,))
        self.half = (float(hs[0]), float(hs[1]))
        self.center = tuple(float(v) for v in props.get("center", (0.0, 0.0, 0.0)))
        self.bsdf = props.get("bsdf", None)
        self.emitter = props.get("emitter", None)
        if self.ground:
            if self.center != (0.0, 0.0, 0.0) or self.half[0] != self.half[1]:
                raise ValueError("the ground rectangle is centred at the origin with equal half sizes")
            if not isinstance(self.bsdf, TwoStateBSDF) or not self.bsdf.textured:
                raise ValueError("the ground rectangle needs a twostate BSDF with a bitmap reflectance")
        elif not isinstance(self.emitter, AreaEmitter):
            raise ValueError("a non-ground rectangle must carry an 'area' emitter")

    def interior_medium(self):
        return None


class SphereShape:
    is_surface_shape = True

    def __init__(self, props: Properties):
        self.center = tuple(float(v) for v in props.get("center", (0.0, 0.0, 0.0)))
        self.radius = float(props.get("radius", 1.0))
        if self.radius <= 0:
            raise ValueError("sphere radius must be positive")
        b = props.get("bsdf", None)
        if isinstance(b, TwoStateBSDF):
            if b.textured:
                raise ValueError("sphere BSDFs must have a constant reflectance")
            self.bsdf = b
        elif isinstance(b, DiffuseBSDF) and b.texture is None:
            self.bsdf = b
        else:
            raise ValueError("spheres need a diffuse (or twostate diffuse) BSDF with constant reflectance")

    def interior_medium(self):
        return None


class SurfaceSceneView:
    """Device view of a scene's surface shapes (one ground, spheres, one light)."""

    def __init__(self, scene):
        grounds = [s for s in scene.shapes() if isinstance(s, RectangleShape) and s.ground]
        lights = [s for s in scene.shapes() if isinstance(s, RectangleShape) and not s.ground]
        self.spheres = [s for s in scene.shapes() if isinstance(s, SphereShape)]
        if len(grounds) != 1 or len(lights) != 1:
            raise RuntimeError("the surface tracer needs exactly one ground rectangle and one area light")
        if len(self.spheres) > 8:
            raise ValueError("at most 8 spheres are supported")
        self.ground, self.light = grounds[0], lights[0]
        self.bsdf: TwoStateBSDF = self.ground.bsdf
        self.device = self.bsdf.new.texture.device
        self._workspace = None

    def c_struct(self) -> _lib.SurfaceScene:
        b = self.bsdf
        th, tw, _ = b.new.texture.data.shape
        if self._workspace is None:
            n = int(_lib.load().rcv_surface_workspace_bytes(tw, th))
            self._workspace = torch.empty(n + 256, dtype=torch.uint8, device=self.device)
        s = _lib.SurfaceScene()
        s.plane_half = self.ground.half[0]
        s.tex_width, s.tex_height = tw, th
        s.tex_old = b.old.texture.data.data_ptr()
        s.tex_new = b.new.texture.data.data_ptr()
        s.num_spheres = len(self.spheres)
        for k, sp in enumerate(self.spheres):
            refl = sp.bsdf.new.value if isinstance(sp.bsdf, TwoStateBSDF) else sp.bsdf.value
            s.spheres[k].center[:] = list(sp.center)
            s.spheres[k].radius = sp.radius
            s.spheres[k].albedo[:] = list(refl)
        s.light_center[:] = list(self.light.center)
        s.light_half[:] = list(self.light.half)
        s.light_radiance[:] = list(self.light.emitter.radiance)
        s.workspace = (self._workspace.data_ptr() + 255) & ~255
        return s

    def prepare(self, stream) -> _lib.SurfaceScene:
        if self.device.type != "cuda":
            raise RuntimeError("rendering requires the scene on a CUDA device")
        s = self.c_struct()
        if self.bsdf._dirty:
            _lib.check(_lib.load().rcv_surface_prepare(C.byref(s), stream), "rcv_surface_prepare")
            self.bsdf._dirty = False
        return s


for _name, _ctor, _kind in [
    ("bitmap", BitmapTexture, "texture"),
    ("area", AreaEmitter, "emitter"),
    ("rectangle", RectangleShape, "shape"),
    ("sphere", SphereShape, "shape"),
]:
    register_object(_kind, _name, _ctor)
register_bsdf("diffuse", DiffuseBSDF)
register_bsdf("twostate", TwoStateBSDF)
