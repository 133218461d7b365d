"""CPU oracle — TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module; the product never does.

Two parts:
  * ctypes access to ``rcv_oracle.cpp`` (the sequential C++ restatement of the
    two-state tracer, the single-state tracer and the path-replay adjoint);
  * a float32-faithful numpy restatement of the control-variate blend and the
    EMA-Welford statistics, following
        plugins/cv_integrator.py:58-77      CVIntegrator.render
        plugins/metaintegrator.py:93-113    MetaIntegrator.render (cv_ps)
        plugins/welford.py:4-78             Welford estimators
    and of the Adam step (Kingma & Ba 2015) used by optimize.py:90,127.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import build as _build

_lib = None


class OracleScene(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("cam_o", C.c_float * 3),
        ("cam_f", C.c_float * 3),
        ("cam_r", C.c_float * 3),
        ("cam_u", C.c_float * 3),
        ("max_depth", C.c_int32),
        ("rr_depth", C.c_int32),
        ("hide_emitters", C.c_int32),
        ("dx", C.c_int32),
        ("dy", C.c_int32),
        ("dz", C.c_int32),
        ("scale", C.c_float),
        ("dens_old", C.c_void_p),
        ("dens_new", C.c_void_p),
        ("alb_old", C.c_void_p),
        ("alb_new", C.c_void_p),
        ("albedo_const", C.c_float * 3),
        ("majorant_factor", C.c_int32),
        ("box_min", C.c_float * 3),
        ("box_size", C.c_float * 3),
        ("n_cams", C.c_int32),
        ("cams", (C.c_float * 12) * 15),
        ("adx", C.c_int32),
        ("ady", C.c_int32),
        ("adz", C.c_int32),
        ("env_w", C.c_int32),
        ("env_h", C.c_int32),
        ("env_scale", C.c_float),
        ("env_texels", C.c_void_p),
    ]


class OracleSurface(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("cam_o", C.c_float * 3),
        ("cam_f", C.c_float * 3),
        ("cam_r", C.c_float * 3),
        ("cam_u", C.c_float * 3),
        ("max_depth", C.c_int32),
        ("rr_depth", C.c_int32),
        ("hide_emitters", C.c_int32),
        ("plane_half", C.c_float),
        ("tex_w", C.c_int32),
        ("tex_h", C.c_int32),
        ("tex_old", C.c_void_p),
        ("tex_new", C.c_void_p),
        ("nspheres", C.c_int32),
        ("spheres", (C.c_float * 7) * 8),
        ("light_c", C.c_float * 3),
        ("light_h", C.c_float * 2),
        ("light_le", C.c_float * 3),
    ]


class SurfaceScene:
    """Surface scene for the oracle; keeps the numpy textures alive."""

    def __init__(self, cam: "Camera", tex_old, tex_new, spheres, light_c, light_h, light_le, plane_half=2.0,
                 max_depth=8, rr_depth=5, hide_emitters=False):
        self.tex_old = np.ascontiguousarray(tex_old, np.float32)
        self.tex_new = np.ascontiguousarray(tex_new, np.float32)
        s = OracleSurface()
        s.width, s.height = cam.width, cam.height
        s.cam_o[:], s.cam_f[:], s.cam_r[:], s.cam_u[:] = cam.origin, cam.forward, cam.right, cam.up
        s.max_depth = max_depth if max_depth >= 0 else 0x7FFFFFFF
        s.rr_depth = rr_depth
        s.hide_emitters = int(hide_emitters)
        s.plane_half = plane_half
        s.tex_h, s.tex_w = self.tex_new.shape[:2]
        s.tex_old = self.tex_old.ctypes.data
        s.tex_new = self.tex_new.ctypes.data
        s.nspheres = len(spheres)
        for k, (c, r, a) in enumerate(spheres):
            s.spheres[k][:] = [float(np.float32(v)) for v in (*c, r, *a)]
        s.light_c[:] = [float(np.float32(v)) for v in light_c]
        s.light_h[:] = [float(np.float32(v)) for v in light_h]
        s.light_le[:] = [float(np.float32(v)) for v in light_le]
        self.c = s
        self.width, self.height = cam.width, cam.height


def surface_render_twostates(scene: SurfaceScene, seed: int, spp: int, threads: int | None = None,
                             rows: tuple = (0, 0, 1)):
    """(H, F); ``rows`` = (first, end[, stride]) rows to render (end 0 = all)."""
    H = np.zeros((scene.height, scene.width, 3), np.float32)
    F = np.zeros_like(H)
    if lib().oracle_surface_render(C.byref(scene.c), 0, seed & 0xFFFFFFFF, spp, H.ctypes.data, F.ctypes.data,
                                   threads or default_threads(), *_rows(rows)):
        raise ValueError("oracle_surface_render: invalid arguments")
    return H, F


def surface_render(scene: SurfaceScene, seed: int, spp: int, threads: int | None = None, rows: tuple = (0, 0, 1)):
    img = np.zeros((scene.height, scene.width, 3), np.float32)
    if lib().oracle_surface_render(C.byref(scene.c), 1, seed & 0xFFFFFFFF, spp, None, img.ctypes.data,
                                   threads or default_threads(), *_rows(rows)):
        raise ValueError("oracle_surface_render: invalid arguments")
    return img


def surface_backward(scene: SurfaceScene, seed: int, spp: int, grad_img, threads: int | None = None,
                     rows: tuple = (0, 0, 1)):
    """dLoss/dtexture (float64) from the paths of the selected rows."""
    g = np.ascontiguousarray(grad_img, np.float32)
    out = np.zeros(scene.tex_new.shape, np.float64)
    if lib().oracle_surface_backward(C.byref(scene.c), seed & 0xFFFFFFFF, spp, g.ctypes.data, out.ctypes.data,
                                     threads or default_threads(), *_rows(rows)):
        raise ValueError("oracle_surface_backward: invalid arguments")
    return out


def surface_forward(scene: SurfaceScene, seed: int, spp: int, tangent, threads: int | None = None):
    """Forward-mode derivative image of the surface render along a texture
    tangent [tex_h][tex_w][3]."""
    t = np.ascontiguousarray(tangent, np.float32)
    out = np.zeros((scene.height, scene.width, 3), np.float32)
    if lib().oracle_surface_forward(C.byref(scene.c), seed & 0xFFFFFFFF, spp, t.ctypes.data, out.ctypes.data,
                                    threads or default_threads()):
        raise ValueError("oracle_surface_forward: invalid arguments")
    return out


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(str(path))
        vp = C.c_void_p
        L.oracle_render.argtypes = [C.POINTER(OracleScene), C.c_int, C.c_uint32, C.c_int, C.c_int, vp, vp, vp, C.c_int,
                                    C.c_int, C.c_int, C.c_int]
        L.oracle_render.restype = C.c_int
        L.oracle_backward.argtypes = [C.POINTER(OracleScene), C.c_uint32, C.c_int, vp, vp, vp, C.c_int, C.c_int,
                                      C.c_int, C.c_int]
        L.oracle_backward.restype = C.c_int
        L.oracle_forward.argtypes = [C.POINTER(OracleScene), C.c_uint32, C.c_int, vp, vp, vp, C.c_int]
        L.oracle_forward.restype = C.c_int
        L.oracle_surface_render.argtypes = [C.POINTER(OracleSurface), C.c_int, C.c_uint32, C.c_int, vp, vp, C.c_int,
                                            C.c_int, C.c_int, C.c_int]
        L.oracle_surface_render.restype = C.c_int
        L.oracle_surface_backward.argtypes = [C.POINTER(OracleSurface), C.c_uint32, C.c_int, vp, vp, C.c_int, C.c_int,
                                              C.c_int, C.c_int]
        L.oracle_surface_forward.argtypes = [C.POINTER(OracleSurface), C.c_uint32, C.c_int, vp, vp, C.c_int]
        L.oracle_surface_forward.restype = C.c_int
        L.oracle_surface_backward.restype = C.c_int
        L.oracle_sample_tea_32.argtypes = [C.c_uint32, C.c_uint32]
        L.oracle_sample_tea_32.restype = C.c_uint32
        L.oracle_pcg32.argtypes = [C.c_uint64, C.c_uint64, C.c_int, vp]
        L.oracle_pcg32.restype = None
        L.oracle_rng_stream.argtypes = [C.c_uint32, C.c_uint32, C.c_int, vp]
        L.oracle_rng_stream.restype = None
        L.oracle_log_unit.argtypes = [vp, C.c_int, vp]
        L.oracle_log_unit.restype = None
        L.oracle_uniform_sphere.argtypes = [vp, C.c_int, vp]
        L.oracle_uniform_sphere.restype = None
        L.oracle_vps_alt_seed.argtypes = [C.c_uint32]
        L.oracle_vps_alt_seed.restype = C.c_uint32
        L.oracle_exp_nonpos.argtypes = [C.c_float]
        L.oracle_exp_nonpos.restype = C.c_float
        L.oracle_vps_render.argtypes = [C.POINTER(OracleScene), vp, C.c_uint32, C.c_int, vp, C.c_int, C.c_int, C.c_int,
                                        C.c_int]
        L.oracle_vps_render.restype = C.c_int
        L.oracle_vps_backward.argtypes = [C.POINTER(OracleScene), vp, C.c_uint32, C.c_int, vp, vp, vp, C.c_int]
        L.oracle_vps_backward.restype = C.c_int
        L.oracle_env_uv.argtypes = [vp, C.c_int, vp]
        L.oracle_env_uv.restype = None
        L.oracle_atan2.argtypes = [C.c_float, C.c_float]
        L.oracle_atan2.restype = C.c_float
        L.oracle_env_sample.argtypes = [C.POINTER(OracleScene), vp, C.c_int, vp, vp, vp]
        L.oracle_env_sample.restype = C.c_int
        L.oracle_env_eval.argtypes = [C.POINTER(OracleScene), vp, C.c_int, vp, vp]
        L.oracle_env_eval.restype = C.c_int
        _lib = L
    return _lib


def default_threads() -> int:
    try:
        return max(1, len(os.sched_getaffinity(0)))
    except AttributeError:  # pragma: no cover
        return max(1, os.cpu_count() or 1)


@dataclass
class Camera:
    width: int
    height: int
    origin: tuple
    forward: tuple
    right: tuple
    up: tuple


def camera_basis(width, height, origin=(0.5, 0.5, 3.5), target=(0.5, 0.5, 0.5), up=(0.0, 1.0, 0.0), fov=45.0):
    """Pinhole basis (float32) for a look-at camera with horizontal fov."""
    o = np.array(origin, np.float64)
    f = np.array(target, np.float64) - o
    f /= np.linalg.norm(f)
    r = np.cross(f, np.array(up, np.float64))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    tx = np.tan(np.radians(fov) * 0.5)
    ty = tx * height / width
    as32 = lambda v: tuple(float(np.float32(x)) for x in v)  # noqa: E731
    return Camera(width, height, as32(o), as32(f), as32(r * tx), as32(u * ty))


class Scene:
    """Keeps the numpy grids alive while the C structure points at them.

    ``cam``: one Camera, or a list of Cameras of equal film size rendering
    side by side into one film (a batch sensor).  ``box_min`` / ``box_size``:
    the medium box, to_world = translate(box_min) * scale(box_size)."""

    def __init__(self, cam, dens_old, dens_new, albedo_old=None, albedo_new=None, albedo_const=0.8,
                 max_depth=16, rr_depth=None, hide_emitters=False, scale=1.0, majorant_factor=0,
                 box_min=(0.0, 0.0, 0.0), box_size=(1.0, 1.0, 1.0), envmap=None, envmap_scale=1.0):
        cams = list(cam) if isinstance(cam, (list, tuple)) else [cam]
        if not 1 <= len(cams) <= 16 or any((c.width, c.height) != (cams[0].width, cams[0].height) for c in cams):
            raise ValueError("a batch film takes 1..16 sub-sensors of one film size")
        cam = Camera(cams[0].width * len(cams), cams[0].height, cams[0].origin, cams[0].forward, cams[0].right,
                     cams[0].up)
        self.dens_old = np.ascontiguousarray(dens_old, np.float32)
        self.dens_new = np.ascontiguousarray(dens_new, np.float32)
        dz, dy, dx = self.dens_new.shape[:3]
        self.alb_old = None if albedo_old is None else np.ascontiguousarray(albedo_old, np.float32)
        self.alb_new = None if albedo_new is None else np.ascontiguousarray(albedo_new, np.float32)
        s = OracleScene()
        s.width, s.height = cam.width, cam.height
        s.cam_o[:], s.cam_f[:], s.cam_r[:], s.cam_u[:] = cam.origin, cam.forward, cam.right, cam.up
        s.max_depth = max_depth if max_depth >= 0 else 0x7FFFFFFF
        s.rr_depth = max_depth if rr_depth is None else rr_depth
        s.hide_emitters = int(hide_emitters)
        s.dx, s.dy, s.dz = dx, dy, dz
        s.scale = scale
        s.dens_old = self.dens_old.ctypes.data
        s.dens_new = self.dens_new.ctypes.data
        s.alb_old = None if self.alb_old is None else self.alb_old.ctypes.data
        s.alb_new = None if self.alb_new is None else self.alb_new.ctypes.data
        ac = np.broadcast_to(np.asarray(albedo_const, np.float32), (3,))
        s.albedo_const[:] = [float(v) for v in ac]
        s.majorant_factor = int(majorant_factor)
        s.box_min[:] = [float(np.float32(v)) for v in box_min]
        s.box_size[:] = [float(np.float32(v)) for v in box_size]
        if self.alb_new is not None and self.alb_new.shape[:3] != (dz, dy, dx):
            s.adz, s.ady, s.adx = self.alb_new.shape[:3]  # the albedo grid's own resolution
        s.n_cams = len(cams)
        for k, c in enumerate(cams[1:]):
            s.cams[k][:] = [*c.origin, *c.forward, *c.right, *c.up]
        # environment map [H][W][3] (None: the constant white environment)
        self.envmap = None if envmap is None else np.ascontiguousarray(envmap, np.float32)
        if self.envmap is not None:
            s.env_h, s.env_w = self.envmap.shape[:2]
            s.env_scale = float(envmap_scale)
            s.env_texels = self.envmap.ctypes.data
        self.c = s
        self.width, self.height = cam.width, cam.height


def _rows(rows):
    """(first, end[, stride]) row selection; end 0 = all rows."""
    r = tuple(int(v) for v in rows)
    return (r[0], r[1], r[2] if len(r) > 2 else 1)


def render_twostates(scene: Scene, seed: int, spp: int, chunk: int | None = None, threads: int | None = None,
                     counters=None, rows: tuple = (0, 0, 1)):
    """(H, F) float32 images.  `chunk` = samples per GPU thread (summation
    order); `rows` = (first, end) row band to render (0, 0 = all)."""
    chunk = spp if chunk is None else chunk
    H = np.zeros((scene.height, scene.width, 3), np.float32)
    F = np.zeros_like(H)
    cnt = np.zeros(4, np.uint64) if counters is None else counters
    rc = lib().oracle_render(C.byref(scene.c), 0, seed & 0xFFFFFFFF, spp, chunk, H.ctypes.data, F.ctypes.data,
                             cnt.ctypes.data, threads or default_threads(), *_rows(rows))
    if rc:
        raise ValueError("oracle_render: invalid arguments")
    return H, F


def render(scene: Scene, seed: int, spp: int, chunk: int | None = None, threads: int | None = None, counters=None,
           rows: tuple = (0, 0, 1)):
    """Single-state image of the `new` parameters."""
    chunk = spp if chunk is None else chunk
    img = np.zeros((scene.height, scene.width, 3), np.float32)
    cnt = np.zeros(4, np.uint64) if counters is None else counters
    rc = lib().oracle_render(C.byref(scene.c), 1, seed & 0xFFFFFFFF, spp, chunk, None, img.ctypes.data,
                             cnt.ctypes.data, threads or default_threads(), *_rows(rows))
    if rc:
        raise ValueError("oracle_render: invalid arguments")
    return img


def backward(scene: Scene, seed: int, spp: int, grad_img, threads: int | None = None, rows: tuple = (0, 0, 1)):
    """(grad_density [dz,dy,dx] float64, grad_albedo [dz,dy,dx,3] or None)."""
    g = np.ascontiguousarray(grad_img, np.float32)
    gd = np.zeros(scene.dens_new.shape[:3], np.float64)
    ga = None if scene.alb_new is None else np.zeros(scene.alb_new.shape[:3] + (3,), np.float64)
    rc = lib().oracle_backward(C.byref(scene.c), seed & 0xFFFFFFFF, spp, g.ctypes.data, gd.ctypes.data,
                               None if ga is None else ga.ctypes.data, threads or default_threads(), *_rows(rows))
    if rc:
        raise ValueError("oracle_backward: invalid arguments")
    return gd, ga


def forward(scene: Scene, seed: int, spp: int, tangent_density=None, tangent_albedo=None,
            threads: int | None = None):
    """Forward-mode derivative image (float32 [H][W][3]) of the single-state
    render along the given tangents."""
    td = None if tangent_density is None else np.ascontiguousarray(tangent_density, np.float32)
    ta = None if tangent_albedo is None else np.ascontiguousarray(tangent_albedo, np.float32)
    out = np.zeros((scene.height, scene.width, 3), np.float32)
    rc = lib().oracle_forward(C.byref(scene.c), seed & 0xFFFFFFFF, spp, None if td is None else td.ctypes.data,
                              None if ta is None else ta.ctypes.data, out.ctypes.data, threads or default_threads())
    if rc:
        raise ValueError("oracle_forward: invalid arguments")
    return out


def sample_tea_32(v0: int, v1: int) -> int:
    return int(lib().oracle_sample_tea_32(v0 & 0xFFFFFFFF, v1 & 0xFFFFFFFF))


def pcg32(initstate: int, initseq: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().oracle_pcg32(initstate, initseq, n, out.ctypes.data)
    return out


def rng_stream(seed: int, lane: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float32)
    lib().oracle_rng_stream(seed & 0xFFFFFFFF, lane & 0xFFFFFFFF, n, out.ctypes.data)
    return out


def log_unit(x) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(x)
    lib().oracle_log_unit(x.ctypes.data, x.size, out.ctypes.data)
    return out


def uniform_sphere(u) -> np.ndarray:
    u = np.ascontiguousarray(u, np.float32).reshape(-1, 2)
    out = np.zeros((u.shape[0], 3), np.float32)
    lib().oracle_uniform_sphere(u.ctypes.data, u.shape[0], out.ctypes.data)
    return out


# --------------------------------------------------------------------------
# float32-faithful restatement of the control variate and Welford statistics
f32 = np.float32


def pow_f32(b: float, n: int) -> np.float32:
    """beta^n of a float32 beta, rounded to float32."""
    return f32(float(f32(b)) ** n)


class StatisticsOracle:
    """plugins/welford.py:38-78 in numpy float32."""

    def __init__(self, beta1=0.9, beta2=0.999):
        self.n = 0
        self.b1 = f32(beta1)
        self.b2 = f32(beta2)
        self.mean_x = self.mean_y = self.var_x = self.var_y = self.cov = f32(0.0)

    def update(self, x, y):
        x = np.asarray(x, f32)
        y = np.asarray(y, f32)
        one = f32(1.0)
        if self.n > 0:
            d = one - pow_f32(self.b1, self.n)
            dx1 = x - (self.mean_x / d).astype(f32)
            dy1 = y - (self.mean_y / d).astype(f32)
        else:
            dx1, dy1 = x, y
        omb1 = one - self.b1
        omb2 = one - self.b2
        self.mean_y = (self.b1 * self.mean_y + omb1 * y).astype(f32)
        self.mean_x = (self.b1 * self.mean_x + omb1 * x).astype(f32)
        self.n += 1
        d = one - pow_f32(self.b1, self.n)
        dx2 = (x - self.mean_x / d).astype(f32)
        dy2 = (y - self.mean_y / d).astype(f32)
        self.var_x = (self.b2 * self.var_x + (omb2 * dx1) * dx2).astype(f32)
        self.var_y = (self.b2 * self.var_y + (omb2 * dy1) * dy2).astype(f32)
        self.cov = (self.b2 * self.cov + (omb2 * dx1) * dy2).astype(f32)

    def get(self):
        d = f32(1.0) - pow_f32(self.b2, self.n)
        return (np.asarray(self.var_x / d, f32), np.asarray(self.var_y / d, f32), np.asarray(self.cov / d, f32))


class WelfordOracle:
    """plugins/welford.py:4-36 in numpy float32."""

    def __init__(self, beta1=0.9, beta2=0.999):
        self.n = 0
        self.b1 = f32(beta1)
        self.b2 = f32(beta2)
        self.mean = f32(0.0)
        self.var = f32(0.0)

    def update(self, x):
        x = np.asarray(x, f32)
        one = f32(1.0)
        if self.n > 0:
            dx1 = (x - self.mean / (one - pow_f32(self.b1, self.n))).astype(f32)
        else:
            dx1 = x
        self.mean = (self.b1 * self.mean + (one - self.b1) * x).astype(f32)
        self.n += 1
        dx2 = (x - self.mean / (one - pow_f32(self.b1, self.n))).astype(f32)
        self.var = (self.b2 * self.var + ((one - self.b2) * dx1) * dx2).astype(f32)

    def get(self):
        return np.asarray(self.var / (f32(1.0) - pow_f32(self.b2, self.n)), f32)


class CVOracle:
    """CVIntegrator.render minus the tracer (plugins/cv_integrator.py:58-77),
    with MetaIntegrator's pre_update option (plugins/metaintegrator.py:95-111)."""

    def __init__(self, warmup=1, beta1=0.9, beta2=0.999, pre_update=False):
        self.warmup = warmup
        self.pre_update = pre_update
        self.stats = StatisticsOracle(beta1, beta2)
        self.img = f32(0.0)
        self.v_n = f32(0.0)
        self.w_s = f32(0.0)
        self.it = 0

    def step(self, H, F):
        H = np.asarray(H, f32)
        F = np.asarray(F, f32)
        if self.it > 0 and self.pre_update:
            self.stats.update(H, F)
        if self.it > self.warmup:
            v0, v1, cov = self.stats.get()
            w = np.asarray(self.w_s, f32)
            self.v_n = ((w * w) * (self.v_n + v0) + v1 - (f32(2.0) * w) * cov).astype(f32)
            with np.errstate(divide="ignore", invalid="ignore"):
                ws = (cov / (v0 + self.v_n)).astype(f32)
            ws = np.where(np.isnan(ws) | np.isinf(ws), f32(0.0), ws).astype(f32)
            self.w_s = np.clip(ws, f32(0.0), f32(1.0)).astype(f32)
        self.img = (self.w_s * (self.img - H) + F).astype(f32)
        if self.it > 0 and not self.pre_update:
            self.stats.update(H, F)
        self.it += 1
        return self.img


class MetaOracle:
    """MetaIntegrator.render (plugins/metaintegrator.py:57-130) around a
    nested integrator given as two callables: ``render_twostates(seed)`` ->
    (H, F) and ``render(seed)`` -> image.  Methods ``baseline``, ``cv_ps``,
    ``cv_pss``; ``pre_update``; ``force_baseline`` (denoising is not
    restated)."""

    def __init__(self, method="baseline", warmup=1, beta1=0.9, beta2=0.999, pre_update=False,
                 force_baseline=False):
        self.method = method
        self.force_baseline = force_baseline
        self.cv = CVOracle(warmup, beta1, beta2, pre_update) if "cv" in method else None
        self.H = f32(0.0)  # cv_pss: the previous step's render with this step's seed
        self.img = f32(0.0)

    def render(self, render_twostates, render, seed):
        img_noisy = None
        if self.method == "cv_ps":
            H, F = render_twostates(seed)
        else:
            img_noisy = render(seed)
        if self.method == "cv_pss":
            H, F = self.H, img_noisy
        if self.cv is not None:
            self.img = self.cv.step(H, F)
        else:
            self.img = img_noisy
        if self.method == "cv_pss":
            self.H = render(seed + 1)  # re-rendered with the next step's seed
        if self.force_baseline:
            return img_noisy if self.method != "cv_ps" else render(seed)
        return self.img


def adam_step(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8, lo=-np.inf, hi=np.inf):
    """One Adam step in float32 arithmetic (bias correction in the step size)."""
    p, g, m, v = (np.asarray(a, f32) for a in (p, g, m, v))
    lr_t = f32(lr * np.sqrt(1.0 - float(f32(b2)) ** t) / (1.0 - float(f32(b1)) ** t))
    b1f, b2f = f32(b1), f32(b2)
    m = (b1f * m + (f32(1.0) - b1f) * g).astype(f32)
    v = (b2f * v + (f32(1.0) - b2f) * (g * g)).astype(f32)
    p = (p - (lr_t * m) / (np.sqrt(v) + f32(eps))).astype(f32)
    p = np.clip(p, f32(lo), f32(hi)).astype(f32)
    return p, m, v


# ------------------------------------------------------------ volpathsimple
VPS_DEFAULT = dict(use_nee=True, use_drt=True, use_drt_subsampling=True, use_drt_mis=True)


def _vps_flags(flags):
    f = dict(VPS_DEFAULT)
    f.update(flags or {})
    return np.array([int(bool(f[k])) for k in ("use_nee", "use_drt", "use_drt_subsampling", "use_drt_mis")],
                    np.int32)


def vps_render(scene: Scene, seed: int, spp: int, flags=None, threads: int | None = None, rows: tuple = (0, 0, 1)):
    """volpathsimple primal image (plugins/volpathsimple.py)."""
    fl = _vps_flags(flags)
    img = np.zeros((scene.height, scene.width, 3), np.float32)
    rc = lib().oracle_vps_render(C.byref(scene.c), fl.ctypes.data, seed & 0xFFFFFFFF, spp, img.ctypes.data,
                                 threads or default_threads(), *_rows(rows))
    if rc:
        raise ValueError("oracle_vps_render: invalid arguments")
    return img


def vps_backward(scene: Scene, seed: int, spp: int, grad_img, flags=None, threads: int | None = None):
    """volpathsimple adjoint: (grad_density float64, grad_albedo or None)."""
    fl = _vps_flags(flags)
    g = np.ascontiguousarray(grad_img, np.float32)
    gd = np.zeros(scene.dens_new.shape[:3], np.float64)
    ga = None if scene.alb_new is None else np.zeros(scene.alb_new.shape[:3] + (3,), np.float64)
    rc = lib().oracle_vps_backward(C.byref(scene.c), fl.ctypes.data, seed & 0xFFFFFFFF, spp, g.ctypes.data,
                                   gd.ctypes.data, None if ga is None else ga.ctypes.data,
                                   threads or default_threads())
    if rc:
        raise ValueError("oracle_vps_backward: invalid arguments")
    return gd, ga


def vps_alt_seed(seed: int) -> int:
    return int(lib().oracle_vps_alt_seed(seed & 0xFFFFFFFF))


def exp_nonpos(x: float) -> float:
    return float(lib().oracle_exp_nonpos(float(x)))


# ------------------------------------------------------- environment map
def env_uv(dirs) -> np.ndarray:
    """(u, v, sin theta) of unit world directions [n][3]."""
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    out = np.zeros((d.shape[0], 3), np.float32)
    lib().oracle_env_uv(d.ctypes.data, d.shape[0], out.ctypes.data)
    return out


def atan2(y: float, x: float) -> float:
    return float(lib().oracle_atan2(float(y), float(x)))


def env_sample(scene: Scene, u) -> tuple:
    """Directions [n][3], radiance [n][3] and pdf [n] sampled from uniforms [n][2]."""
    u = np.ascontiguousarray(u, np.float32).reshape(-1, 2)
    n = u.shape[0]
    d, le, pdf = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32), np.zeros(n, np.float32)
    if lib().oracle_env_sample(C.byref(scene.c), u.ctypes.data, n, d.ctypes.data, le.ctypes.data, pdf.ctypes.data):
        raise ValueError("oracle_env_sample: the scene has no environment map")
    return d, le, pdf


def env_eval(scene: Scene, dirs) -> tuple:
    """Radiance [n][3] and sampling pdf [n] of the map along unit directions."""
    d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    n = d.shape[0]
    le, pdf = np.zeros((n, 3), np.float32), np.zeros(n, np.float32)
    if lib().oracle_env_eval(C.byref(scene.c), d.ctypes.data, n, le.ctypes.data, pdf.ctypes.data):
        raise ValueError("oracle_env_eval: the scene has no environment map")
    return le, pdf
