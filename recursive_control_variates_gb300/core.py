"""Scene description objects, the plugin registry and scene parameters.

This mirrors the part of Mitsuba's plugin system the reference path uses:
``mi.load_dict`` over nested ``{'type': name, ...}`` dictionaries
(optimize.py:66, experiments.py:20-132), ``mi.register_integrator / bsdf /
medium`` (plugins/__init__.py:11-17), and ``mi.traverse(scene)`` with
``params.update(opt)`` (optimize.py:41,107).

Supported scene family (the synthetic configurations of this project): one
unit-cube shape ``[0,1]^3`` with a ``null`` BSDF whose interior is a
(two-state) heterogeneous medium, a ``constant`` environment emitter of
radiance 1, a ``perspective`` sensor with an ``hdrfilm`` and a ``box``
reconstruction filter.  Anything else raises ``ValueError`` at load time.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Any, Callable

import numpy as np
import torch

from . import _lib

# ----------------------------------------------------------------- registry
_REGISTRY: dict[str, Callable[["Properties"], Any]] = {}
_KINDS: dict[str, str] = {}


def _register(kind: str, name: str, ctor: Callable[["Properties"], Any]) -> None:
    _REGISTRY[name] = ctor
    _KINDS[name] = kind


def register_integrator(name: str, ctor) -> None:
    _register("integrator", name, ctor)


def register_bsdf(name: str, ctor) -> None:
    _register("bsdf", name, ctor)


def register_medium(name: str, ctor) -> None:
    _register("medium", name, ctor)


def register_object(kind: str, name: str, ctor) -> None:
    _register(kind, name, ctor)


class Properties(dict):
    """Plugin properties: a dict with Mitsuba's ``props.get`` / ``props[key]``."""

    def __init__(self, plugin: str, values: dict):
        super().__init__(values)
        self.plugin = plugin

    def __getitem__(self, key):
        if key not in self:
            raise KeyError(f"plugin '{self.plugin}': required property '{key}' is missing")
        return super().__getitem__(key)


def load_dict(d: dict, device: str | torch.device | None = None) -> Any:
    """Instantiates a plugin tree (``mi.load_dict`` equivalent)."""
    if not isinstance(d, dict):
        raise TypeError("load_dict expects a dictionary")
    if "type" not in d:
        raise ValueError("missing 'type' entry")
    name = d["type"]
    if name not in _REGISTRY:
        raise ValueError(f"unknown plugin type '{name}'")
    values = {}
    for k, v in d.items():
        if k == "type":
            continue
        if isinstance(v, dict) and "type" in v:
            v = load_dict(v, device)
        values[k] = v
    if device is not None:
        values.setdefault("device", device)
    return _REGISTRY[name](Properties(name, values))


def _device(props: Properties) -> torch.device:
    return torch.device(props.get("device", "cuda"))


# -------------------------------------------------------------- transforms
@dataclass(frozen=True)
class LookAt:
    origin: tuple
    target: tuple
    up: tuple


def look_at(origin, target, up) -> LookAt:
    """``T.look_at(origin=..., target=..., up=...)`` of the scene dictionaries."""
    return LookAt(tuple(map(float, origin)), tuple(map(float, target)), tuple(map(float, up)))


@dataclass(frozen=True)
class BoxTransform:
    """Axis-aligned affine map x -> scale * x + translate (positive scale):
    the ``to_world`` of the reference's medium boxes, ``T.scale(s)`` and
    ``T.translate(t).scale(s)`` (experiments.py:57,64,79,285).  Composes like
    Mitsuba's transforms: ``a.scale(s)`` is the product a * scale(s), so
    ``T.translate(t).scale(s)`` maps x to t + s x."""

    scale_: tuple = (1.0, 1.0, 1.0)
    translate_: tuple = (0.0, 0.0, 0.0)

    def __post_init__(self):
        if any(not (v > 0 and math.isfinite(v)) for v in self.scale_):
            raise ValueError("box transforms need a positive, finite scale")

    def __matmul__(self, other: "BoxTransform") -> "BoxTransform":
        s = tuple(a * b for a, b in zip(self.scale_, other.scale_))
        t = tuple(a * b + c for a, b, c in zip(self.scale_, other.translate_, self.translate_))
        return BoxTransform(s, t)

    def scale(self, v) -> "BoxTransform":
        return self @ T.scale(v)

    def translate(self, v) -> "BoxTransform":
        return self @ T.translate(v)

    @property
    def box_min(self) -> tuple:
        return self.translate_

    @property
    def box_size(self) -> tuple:
        return self.scale_


def _vec3(v) -> tuple:
    a = np.broadcast_to(np.asarray(v, np.float64), (3,))
    return tuple(float(x) for x in a)


class T:
    """``mitsuba.scalar_rgb.Transform4f`` as the reference's scene
    dictionaries use it: ``T.look_at(origin=, target=, up=)`` for sensors,
    ``T.scale(s)`` / ``T.translate(t)`` (chained) for the medium box."""

    @staticmethod
    def look_at(origin, target, up) -> LookAt:
        return look_at(origin, target, up)

    @staticmethod
    def scale(v) -> BoxTransform:
        return BoxTransform(_vec3(v), (0.0, 0.0, 0.0))

    @staticmethod
    def translate(v) -> BoxTransform:
        return BoxTransform((1.0, 1.0, 1.0), _vec3(v))


UNIT_BOX = BoxTransform()


# ------------------------------------------------------------------ sensors
class Film:
    def __init__(self, props: Properties):
        self.width = int(props.get("width", 768))
        self.height = int(props.get("height", 576))
        rf = props.get("rfilter", None)
        if rf is not None and not isinstance(rf, BoxFilter):
            raise ValueError("only the 'box' reconstruction filter is supported")
        if self.width <= 0 or self.height <= 0:
            raise ValueError("film size must be positive")

    def size(self):
        return (self.width, self.height)


class BoxFilter:
    def __init__(self, props: Properties):
        pass


class IndependentSampler:
    def __init__(self, props: Properties):
        self.sample_count = int(props.get("sample_count", 4))


class PerspectiveSensor:
    """Pinhole camera; ``fov`` is the horizontal field of view in degrees."""

    def __init__(self, props: Properties):
        self.fov = float(props.get("fov", 45.0))
        if props.get("fov_axis", "x") != "x":
            raise ValueError("only fov_axis='x' is supported")
        tw = props.get("to_world", look_at((0, 0, 0), (0, 0, 1), (0, 1, 0)))
        if not isinstance(tw, LookAt):
            raise ValueError("sensor to_world must be a look_at transform")
        self.to_world = tw
        self.film_ = props.get("film", None) or Film(Properties("hdrfilm", {}))
        self.sampler_ = props.get("sampler", None) or IndependentSampler(Properties("independent", {}))

    def film(self) -> Film:
        return self.film_

    def sampler(self):
        return self.sampler_

    def frame(self, width: int, height: int) -> tuple:
        """(origin, forward, right * tan(fov/2), up * tan(fov/2) * h / w) as
        float32 values, for a film of width x height (memoised: every render
        call asks for it)."""
        key = (width, height, self.fov, self.to_world)
        cache = self.__dict__.setdefault("_frames", {})
        if key not in cache:
            cache[key] = self._frame(width, height)
        return cache[key]

    def _frame(self, width: int, height: int) -> tuple:
        o = np.array(self.to_world.origin, np.float64)
        t = np.array(self.to_world.target, np.float64)
        up = np.array(self.to_world.up, np.float64)
        fwd = t - o
        fwd /= np.linalg.norm(fwd)
        right = np.cross(fwd, up)
        right /= np.linalg.norm(right)
        cam_up = np.cross(right, fwd)
        tx = math.tan(math.radians(self.fov) * 0.5)
        ty = tx * height / width
        f32 = lambda v: tuple(float(np.float32(x)) for x in v)  # noqa: E731
        return f32(o), f32(fwd), f32(right * tx), f32(cam_up * ty)

    def c_struct(self) -> _lib.Sensor:
        w, h = self.film_.width, self.film_.height
        s = _lib.Sensor()
        s.width, s.height = w, h
        s.origin[:], s.forward[:], s.right[:], s.up[:] = self.frame(w, h)
        s.count = 1
        return s


class BatchSensor:
    """``batch`` (Mitsuba's batch sensor; every grid scene of the reference,
    experiments.py:28-50,141-164,257-281): the perspective sub-sensors of the
    dictionary render side by side into one film of width n * w; sub-sensor k
    sees pixels [k w, (k+1) w) with a film of w x height.  Sub-sensors are
    taken in dictionary order."""

    def __init__(self, props: Properties):
        self.film_ = props.get("film", None) or Film(Properties("hdrfilm", {}))
        self.sampler_ = props.get("sampler", None) or IndependentSampler(Properties("independent", {}))
        self.sensors = [v for v in props.values() if isinstance(v, PerspectiveSensor)]
        n = len(self.sensors)
        if not 1 <= n <= _lib.MAX_SENSORS:
            raise ValueError(f"a batch sensor takes 1..{_lib.MAX_SENSORS} perspective sensors, got {n}")
        if self.film_.width % n:
            raise ValueError(f"batch film width {self.film_.width} is not a multiple of its {n} sensors")

    def film(self) -> Film:
        return self.film_

    def sampler(self):
        return self.sampler_

    def c_struct(self) -> _lib.Sensor:
        n = len(self.sensors)
        w, h = self.film_.width, self.film_.height
        sub_w = w // n
        s = _lib.Sensor()
        s.width, s.height = w, h
        s.origin[:], s.forward[:], s.right[:], s.up[:] = self.sensors[0].frame(sub_w, h)
        s.count = n
        for k, sub in enumerate(self.sensors[1:]):
            f = s.more[k]
            f.origin[:], f.forward[:], f.right[:], f.up[:] = sub.frame(sub_w, h)
        return s


# ----------------------------------------------------------------- emitters
class ConstantEmitter:
    def __init__(self, props: Properties):
        rad = props.get("radiance", 1.0)
        if isinstance(rad, dict):
            rad = rad.get("value", 1.0)
        arr = np.broadcast_to(np.asarray(rad, np.float64), (3,))
        if not np.allclose(arr, 1.0):
            raise ValueError("the constant emitter supports radiance 1.0 only")


class EnvmapEmitter:
    """``envmap`` (the reference's grid scenes light the medium with one,
    experiments.py:81-85,195-199,315-319): a latitude-longitude RGB image of
    linear radiance from ``filename`` (OpenEXR) or ``data`` ((H, W, 3)), times
    ``scale``.  Row 0 is the +y pole; a direction (x, y, z) reads the image at
    u = atan2(x, -z) / (2 pi), v = acos(y) / pi, bilinearly.  NEE samples
    it by importance (luminance x sin(theta)).  Only the identity
    ``to_world`` is supported."""

    def __init__(self, props: Properties):
        from . import io

        if props.get("to_world") is not None:
            raise ValueError("envmap: only the identity to_world is supported")
        data = props.get("data")
        if data is None:
            fn = props.get("filename")
            if fn is None:
                raise ValueError("envmap: 'filename' or 'data' is required")
            data = io.read_exr(fn)
        arr = data if isinstance(data, torch.Tensor) else torch.as_tensor(np.asarray(data, np.float32))
        if arr.dim() == 2:
            arr = arr[..., None].expand(-1, -1, 3)
        if arr.dim() != 3 or arr.shape[2] not in (1, 3, 4):
            raise ValueError(f"envmap: expected an (H, W, 3) image, got shape {tuple(arr.shape)}")
        if arr.shape[2] == 1:
            arr = arr.expand(-1, -1, 3)
        arr = arr[..., :3]
        self.scale = float(props.get("scale", 1.0))
        if not np.isfinite(self.scale) or self.scale < 0.0:
            raise ValueError("envmap: scale must be finite and >= 0")
        self.device = _device(props)
        self.texels = arr.detach().to(device=self.device, dtype=torch.float32).contiguous().clone()
        if not bool(torch.isfinite(self.texels).all()) or float(self.texels.min()) < 0.0:
            raise ValueError("envmap: radiance must be finite and non-negative")
        self.height, self.width = int(self.texels.shape[0]), int(self.texels.shape[1])
        self._struct = None
        self._ws = None
        if self.device.type == "cuda":
            self.prepare()

    def prepare(self, stream=None):
        """(Re)builds the sampling tables on the device after the texels change."""
        from .utils import stream_handle

        lib = _lib.load()
        need = int(lib.rcv_envmap_workspace_bytes(self.width, self.height)) + 256
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        s = _lib.Envmap()
        s.width, s.height, s.scale = self.width, self.height, self.scale
        s.texels = self.texels.data_ptr()
        s.workspace = (self._ws.data_ptr() + 255) & ~255
        _lib.check(lib.rcv_envmap_prepare(C.byref(s), stream if stream is not None else stream_handle(self.device)),
                   "rcv_envmap_prepare")
        self._struct = s

    def c_struct(self) -> "_lib.Envmap":
        if self._struct is None:
            raise RuntimeError("envmap: tables not prepared (a CUDA device is required)")
        return self._struct


# ------------------------------------------------------------------- media
class Isotropic:
    def __init__(self, props: Properties):
        pass


def _as_tensor(x, device, channels: int) -> torch.Tensor:
    t = torch.as_tensor(np.asarray(x) if not isinstance(x, torch.Tensor) else x)
    # own copy: the states of a two-state object must never alias each other
    t = t.detach().to(device=device, dtype=torch.float32).clone().contiguous()
    if t.dim() == 3:
        t = t.unsqueeze(-1)
    if t.dim() != 4 or t.shape[-1] != channels:
        raise ValueError(f"grid data must have shape (Dz, Dy, Dx, {channels}), got {tuple(t.shape)}")
    return t


class GridVolume:
    """``gridvolume``: in-memory ``data`` of shape (Dz, Dy, Dx, C) or a
    ``.vol`` ``filename``.  The grid spans ``to_world`` applied to the unit
    cube (``use_grid_bbox``: the bounding box stored in the file instead).
    ``accel`` only selects Mitsuba's texture path and changes nothing here."""

    def __init__(self, props: Properties):
        self.device = _device(props)
        to_world = props.get("to_world", UNIT_BOX)
        if not isinstance(to_world, BoxTransform):
            raise ValueError("gridvolume to_world must be an axis-aligned scale/translate (T.scale, T.translate)")
        if "filename" in props:
            from .io import read_vol

            g = read_vol(props["filename"])
            self.raw = g.data
            if props.get("use_grid_bbox", False):
                size = tuple(b - a for a, b in zip(g.bbox_min, g.bbox_max))
                to_world = to_world @ BoxTransform(size, tuple(g.bbox_min))
        else:
            self.raw = props["data"]
        self.to_world = to_world


class _PackedMedium:
    """Device workspace (packed lookup cells, majorants, gradient
    accumulators) shared by single- and two-state media."""

    _workspace: torch.Tensor | None = None

    # `_dirty`: the grids changed since the last pack.  Setting it also bumps
    # `version`, which tells an adjoint pass started ahead of time whether
    # the parameters it traced are still current.
    @property
    def _dirty(self) -> bool:
        return self.__dict__.get("_dirty_flag", True)

    @_dirty.setter
    def _dirty(self, value: bool) -> None:
        if value:
            self.__dict__["_version"] = self.version + 1
        self.__dict__["_dirty_flag"] = bool(value)

    @property
    def version(self) -> int:
        return self.__dict__.get("_version", 0)

    def add_reader(self, event) -> None:
        """A CUDA event after which work on another stream stops reading the
        workspace; repacking or replacing the workspace waits for it."""
        self.__dict__.setdefault("_readers", []).append(event)

    def _wait_readers(self) -> None:
        readers = self.__dict__.pop("_readers", [])
        if readers:
            s = torch.cuda.current_stream(self.device)
            for ev in readers:
                s.wait_event(ev)

    def _states(self):
        raise NotImplementedError

    def majorant_resolution_factor(self) -> int:
        return self._factor()

    def set_majorant_resolution_factor(self, factor: int) -> None:
        """Supergrid resolution factor (plugins/twostatemedium.py:171-178,
        utils.py:27-43); 0 = one global majorant."""
        if int(factor) < 0:
            raise ValueError("majorant_resolution_factor must be >= 0")
        for m in self._media():
            m.majorant_factor = int(factor)
        self._wait_readers()
        self._workspace = None
        self._dirty = True

    def _media(self):
        return (self,)

    def _factor(self) -> int:
        return self._states()[1].majorant_factor

    def workspace(self) -> torch.Tensor:
        if self._workspace is None:
            m = self._describe(0)
            nbytes = int(_lib.load().rcv_medium_workspace_bytes_for(C.byref(m)))
            if nbytes <= 0:
                raise ValueError("invalid medium description")
            self._workspace = torch.empty(nbytes + 256, dtype=torch.uint8, device=self.device)
        return self._workspace

    @property
    def albedo_dims(self):
        g = self._states()[1].albedo_grid
        if g is None:
            return self.dims
        dz, dy, dx, _ = g.shape
        return (dx, dy, dz)

    def albedo_grad_buffer(self):
        """Zeroed (Dz, Dy, Dx, 3) gradient of the albedo grid, or None."""
        if not self.has_albedo_grid:
            return None
        ax, ay, az = self.albedo_dims
        return torch.zeros((az, ay, ax, 3), dtype=torch.float32, device=self.device)

    def c_struct(self) -> _lib.Medium:
        ws = self.workspace()
        return self._describe((ws.data_ptr() + 255) & ~255)

    def _describe(self, aligned: int) -> _lib.Medium:
        old, new = self._states()
        m = _lib.Medium()
        m.dims[:] = list(self.dims)
        m.scale = new.scale
        m.density_old = old.density.data_ptr()
        m.density_new = new.density.data_ptr()
        if self.has_albedo_grid:
            m.albedo_old = old.albedo_grid.data_ptr()
            m.albedo_new = new.albedo_grid.data_ptr()
        m.albedo_value[:] = list(new.albedo_value)
        m.majorant_factor = self._factor()
        m.workspace = aligned
        m.box_min[:] = [float(np.float32(v)) for v in new.box.box_min]
        m.box_size[:] = [float(np.float32(v)) for v in new.box.box_size]
        if self.has_albedo_grid and tuple(self.albedo_dims) != tuple(self.dims):
            m.albedo_dims[:] = list(self.albedo_dims)
        return m

    def prepare(self, stream) -> _lib.Medium:
        """Packs the grids for the tracers when a state changed."""
        if self.device.type != "cuda":
            raise RuntimeError("rendering requires the medium on a CUDA device")
        m = self.c_struct()
        if self._dirty:
            self._wait_readers()
            _lib.check(_lib.load().rcv_medium_prepare(C.byref(m), stream), "rcv_medium_prepare")
            self._dirty = False
        return m


class HeterogeneousMedium(_PackedMedium):
    """Heterogeneous medium: sigma_t = scale * density grid, albedo constant,
    RGB or grid, isotropic phase function.  Used on its own (single state,
    old = new) or as a state of a ``twostatemedium``."""

    def __init__(self, props: Properties):
        self.device = _device(props)
        st = props["sigma_t"]
        if not isinstance(st, GridVolume):
            raise ValueError("sigma_t must be a gridvolume")
        self.density = _as_tensor(st.raw, self.device, 1)
        self.box = st.to_world
        alb = props.get("albedo", 0.75)
        self.albedo_grid = None
        self.albedo_value = (0.75, 0.75, 0.75)
        if isinstance(alb, GridVolume):
            # the albedo grid may have its own resolution (experiments.py:56,63)
            self.albedo_grid = _as_tensor(alb.raw, self.device, 3)
            if alb.to_world != self.box:
                raise ValueError("albedo and sigma_t grids must have the same to_world")
        else:
            if isinstance(alb, dict):
                alb = alb.get("value", 0.75)
            a = np.broadcast_to(np.asarray(alb, np.float64), (3,))
            self.albedo_value = tuple(float(np.float32(v)) for v in a)
        self.scale = float(props.get("scale", 1.0))
        if self.scale < 0:
            raise ValueError("scale must be non-negative")
        ph = props.get("phase", None)
        if ph is not None and not isinstance(ph, Isotropic):
            raise ValueError("only the isotropic phase function is supported")
        if props.get("has_spectral_extinction", False):
            raise ValueError("spectrally varying extinction is not supported")
        # majorant supergrid of ceil(D/f) cells per axis (0: one global majorant)
        self.majorant_factor = int(props.get("majorant_resolution_factor", 0))
        if self.majorant_factor < 0:
            raise ValueError("majorant_resolution_factor must be >= 0")
        self._workspace = None
        self._dirty = True

    def _states(self):
        return self, self

    @property
    def dims(self):
        dz, dy, dx, _ = self.density.shape
        return (dx, dy, dz)

    @property
    def has_albedo_grid(self) -> bool:
        return self.albedo_grid is not None

    def param_tensors(self) -> dict[str, torch.Tensor]:
        out = {"sigma_t.data": self.density}
        if self.albedo_grid is not None:
            out["albedo.data"] = self.albedo_grid
        return out

    def traverse(self) -> dict[str, torch.Tensor]:
        return self.param_tensors()

    def set_grid(self, sub: str, value: torch.Tensor) -> None:
        """Replaces a grid by one of another resolution (utils.upsample,
        utils.py:177-192, hands the optimiser a finer grid)."""
        t = _as_tensor(value, self.device, 1 if sub == "sigma_t.data" else 3)
        if sub == "sigma_t.data":
            self.density = t
        elif sub == "albedo.data" and self.albedo_grid is not None:
            self.albedo_grid = t
        else:
            raise KeyError(sub)
        self._wait_readers()
        self._workspace = None
        self._dirty = True

    def parameters_changed(self, keys=None) -> None:
        self._dirty = True


class TwoStateMedium(_PackedMedium):
    """Old / new / incoming copies of a heterogeneous medium
    (plugins/twostatemedium.py:5-13).  ``traverse`` exposes ``incoming`` only
    (:186-187); ``parameters_changed`` rotates old <- new <- incoming
    (:189-200) by swapping buffers plus one device copy, then marks the
    lookup workspace for repacking."""

    def __init__(self, props: Properties):
        self.old = props["old"]
        self.new = props["new"]
        self.incoming = props["incoming"]
        for m in (self.old, self.new, self.incoming):
            if not isinstance(m, HeterogeneousMedium):
                raise ValueError("twostatemedium expects heterogeneous media for old/new/incoming")
        if not (self.old.dims == self.new.dims == self.incoming.dims):
            raise ValueError("old/new/incoming grids must have the same resolution")
        if not (self.old.box == self.new.box == self.incoming.box):
            raise ValueError("old/new/incoming grids must have the same to_world")
        if self.new.albedo_grid is not None and not (
                self.old.albedo_grid.shape == self.new.albedo_grid.shape == self.incoming.albedo_grid.shape):
            raise ValueError("old/new/incoming albedo grids must have the same resolution")
        if (self.old.albedo_grid is None) != (self.new.albedo_grid is None) or (
            self.new.albedo_grid is None
        ) != (self.incoming.albedo_grid is None):
            raise ValueError("old/new/incoming must all have, or all lack, an albedo grid")
        self.device = self.new.device
        self._workspace = None
        self._dirty = True

    def _states(self):
        return self.old, self.new

    def _media(self):
        return (self.old, self.new, self.incoming)

    @property
    def dims(self):
        return self.new.dims

    @property
    def has_albedo_grid(self) -> bool:
        return self.new.albedo_grid is not None

    def traverse(self) -> dict[str, torch.Tensor]:
        return self.incoming.param_tensors()

    def set_grid(self, sub: str, value: torch.Tensor) -> None:
        """A new resolution for all three states (utils.upsample).  The
        rotation that follows makes old = new = the new grid; the integrators
        are reset with the upsampling (utils.py:190), so their first step
        does not use the old state's image."""
        for m in (self.old, self.new, self.incoming):
            m.set_grid(sub, value)
        self._wait_readers()
        self._workspace = None
        self._dirty = True

    def parameters_changed(self, keys=None) -> None:
        o, n, i = self.old, self.new, self.incoming
        o.density, n.density = n.density, o.density
        n.density.copy_(i.density)
        if n.albedo_grid is not None:
            o.albedo_grid, n.albedo_grid = n.albedo_grid, o.albedo_grid
            n.albedo_grid.copy_(i.albedo_grid)
        o.albedo_value, n.albedo_value = n.albedo_value, i.albedo_value
        self._dirty = True


class NullBSDF:
    def __init__(self, props: Properties):
        pass


def _check_unit_cube_mesh(path) -> None:
    """The reference bounds its media with common/meshes/cube_unit.obj; any
    OBJ whose vertices are the corners of [0,1]^3 is accepted."""
    verts = []
    with open(path) as f:
        for line in f:
            if line.startswith("v "):
                verts.append([float(x) for x in line.split()[1:4]])
    v = np.array(verts, np.float64)
    if v.size == 0 or not np.all(np.isclose(v, 0.0) | np.isclose(v, 1.0)) or \
            not np.allclose(v.min(axis=0), 0.0) or not np.allclose(v.max(axis=0), 1.0):
        raise ValueError(f"{path}: the medium boundary must be the unit-cube mesh (corners of [0,1]^3)")


class CubeShape:
    """Medium boundary: the unit cube [0,1]^3 (the 'cube_unit' mesh of the
    reference scenes) mapped by ``to_world`` (an axis-aligned scale and
    translation, experiments.py:79,285).  Registered as ``cube`` and as
    ``obj`` (whose ``filename`` must hold the unit-cube mesh)."""

    def __init__(self, props: Properties):
        bsdf = props.get("bsdf", None)
        if bsdf is not None and not isinstance(bsdf, NullBSDF):
            raise ValueError("the medium boundary must use a 'null' BSDF")
        self.to_world = props.get("to_world", UNIT_BOX)
        if not isinstance(self.to_world, BoxTransform):
            raise ValueError("the medium boundary's to_world must be an axis-aligned scale/translate")
        if "filename" in props:
            _check_unit_cube_mesh(props["filename"])
        self.interior = props.get("interior", None)
        med = self.interior
        if med is not None and hasattr(med, "dims"):
            box = med.new.box if hasattr(med, "new") else med.box
            if box != self.to_world:
                raise ValueError("the medium's grids and its boundary shape must have the same to_world")

    def interior_medium(self):
        return self.interior

    def exterior_medium(self):
        return None


class Scene:
    def __init__(self, props: Properties):
        self.sensors_ = []
        self.emitters_ = []
        self.shapes_ = {}
        for k, v in props.items():
            if k == "device":
                continue
            if isinstance(v, (PerspectiveSensor, BatchSensor)):
                self.sensors_.append(v)
            elif isinstance(v, (ConstantEmitter, EnvmapEmitter)):
                self.emitters_.append(v)
            elif isinstance(v, CubeShape) or hasattr(v, "is_surface_shape"):
                self.shapes_[k] = v
            else:
                raise ValueError(f"unsupported scene element '{k}' ({type(v).__name__})")

    def sensors(self):
        return self.sensors_

    def emitters(self):
        return self.emitters_

    def envmap(self):
        """The scene's environment map, or None (constant environment)."""
        env = [e for e in self.emitters_ if isinstance(e, EnvmapEmitter)]
        if len(env) > 1:
            raise ValueError("a scene takes at most one envmap")
        if env and any(isinstance(e, ConstantEmitter) for e in self.emitters_):
            raise ValueError("a scene takes either a constant emitter or an envmap")
        return env[0] if env else None

    def shapes(self):
        return list(self.shapes_.values())

    def named_shapes(self):
        return dict(self.shapes_)


# ------------------------------------------------------- scene parameters
class SceneParameters:
    """``mi.traverse(scene)``: differentiable parameters by key.

    ``params[key] = value`` stages a new value; ``params.update(opt)`` takes
    every key the optimizer holds, copies the values into the scene
    (``incoming`` of a two-state object) and notifies the owners, which
    rotates their states."""

    def __init__(self, scene: Scene):
        self._owners: dict[str, tuple[Any, str]] = {}
        self._values: dict[str, torch.Tensor] = {}
        self._pending: set[str] = set()
        for name, shape in scene.named_shapes().items():
            owners = []
            med = shape.interior_medium() if hasattr(shape, "interior_medium") else None
            if med is not None and hasattr(med, "traverse"):
                owners.append(("interior_medium", med))
            bsdf = getattr(shape, "bsdf", None)
            if bsdf is not None and hasattr(bsdf, "traverse"):
                owners.append(("bsdf", bsdf))
            for prefix, owner in owners:
                for sub, t in owner.traverse().items():
                    key = f"{name}.{prefix}.{sub}"
                    self._owners[key] = (owner, sub)
                    self._values[key] = t

    def keys(self):
        return self._values.keys()

    def items(self):
        return self._values.items()

    def __contains__(self, key):
        return key in self._values

    def __getitem__(self, key):
        return self._values[key]

    def __setitem__(self, key, value):
        if key not in self._owners:
            raise KeyError(f"unknown scene parameter '{key}'")
        owner, sub = self._owners[key]
        cur = owner.traverse()[sub] if hasattr(owner, "traverse") else None
        v = value if isinstance(value, torch.Tensor) else torch.as_tensor(np.asarray(value, np.float32))
        if cur is not None and tuple(v.shape) != tuple(cur.shape):
            if v.numel() == 1:
                v = v.reshape(()).expand(cur.shape)
            elif not (hasattr(owner, "set_grid") and v.dim() == cur.dim() == 4 and v.shape[-1] == cur.shape[-1]):
                raise ValueError(f"parameter '{key}' has shape {tuple(cur.shape)}, got {tuple(v.shape)}")
        self._values[key] = v
        self._pending.add(key)

    def update(self, opt=None):
        if opt is not None:
            for key in opt.keys():
                if key in self._owners:
                    self[key] = opt[key]
        owners = {}
        for key in self._pending:
            owner, sub = self._owners[key]
            dst = owner.traverse()[sub]
            val = self._values[key].detach()
            with torch.no_grad():
                if tuple(val.shape) != tuple(dst.shape) and val.numel() != dst.numel():
                    owner.set_grid(sub, val)  # a new resolution
                else:
                    dst.copy_(val.to(dst.device, torch.float32).reshape(dst.shape))
            owners[id(owner)] = owner
        self._pending.clear()
        for owner in owners.values():
            owner.parameters_changed()
        return self

    def differentiable(self) -> dict[str, torch.Tensor]:
        """Values that take part in differentiation: tensors that require a
        gradient (reverse mode) or carry a forward-mode tangent."""
        from torch.autograd import forward_ad

        def tracked(v):
            return v.requires_grad or forward_ad.unpack_dual(v).tangent is not None

        return {k: v for k, v in self._values.items() if isinstance(v, torch.Tensor) and tracked(v)}

    def owner_of(self, key):
        return self._owners[key]


def traverse(scene: Scene) -> SceneParameters:
    return SceneParameters(scene)


for _name, _ctor, _kind in [
    ("scene", Scene, "scene"),
    ("perspective", PerspectiveSensor, "sensor"),
    ("batch", BatchSensor, "sensor"),
    ("hdrfilm", Film, "film"),
    ("box", BoxFilter, "rfilter"),
    ("independent", IndependentSampler, "sampler"),
    ("constant", ConstantEmitter, "emitter"),
    ("envmap", EnvmapEmitter, "emitter"),
    ("gridvolume", GridVolume, "volume"),
    ("isotropic", Isotropic, "phase"),
    ("heterogeneous", HeterogeneousMedium, "medium"),
    ("null", NullBSDF, "bsdf"),
    ("cube", CubeShape, "shape"),
    ("obj", CubeShape, "shape"),
]:
    register_object(_kind, _name, _ctor)
register_medium("twostatemedium", TwoStateMedium)
