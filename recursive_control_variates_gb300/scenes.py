"""Synthetic scenes of the benchmark configurations.

The reference's own scenes (janga, dust_devil, rover, ...) are separate
downloads that are not available; these seeded generators stand in for them
with the same structure as the reference's grid scenes (experiments.py:20-132):
a unit cube with a null BSDF holding a heterogeneous medium, seen by a
perspective camera, lit by a constant environment.

Density at voxel centres (i+1/2)/D:
    rho(x) = sum_{k<8} a_k exp(-|x - c_k|^2 / (2 s_k^2)),
    c_k ~ U[0.2, 0.8]^3, s_k ~ U[0.05, 0.15], a_k ~ U[5, 20]
drawn from numpy.random.default_rng(seed).  RGB albedo grids are U[0.3, 0.95]
per voxel smoothed by a Gaussian of 2 voxels.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .core import look_at

CAMERA_ORIGIN = (0.5, 0.5, 3.5)
CAMERA_TARGET = (0.5, 0.5, 0.5)
CAMERA_UP = (0.0, 1.0, 0.0)


def blob_density(D: int, seed: int, n_blobs: int = 8) -> np.ndarray:
    """(D, D, D, 1) float32 sum of isotropic Gaussian blobs."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.2, 0.8, size=(n_blobs, 3))
    sigmas = rng.uniform(0.05, 0.15, size=n_blobs)
    amps = rng.uniform(5.0, 20.0, size=n_blobs)
    c = (np.arange(D, dtype=np.float64) + 0.5) / D
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    rho = np.zeros((D, D, D), np.float64)
    for k in range(n_blobs):
        d2 = (x - centres[k, 0]) ** 2 + (y - centres[k, 1]) ** 2 + (z - centres[k, 2]) ** 2
        rho += amps[k] * np.exp(-d2 / (2.0 * sigmas[k] ** 2))
    return rho.astype(np.float32)[..., None]


def albedo_grid(D: int, seed: int, lo: float = 0.3, hi: float = 0.95, smooth: float = 2.0) -> np.ndarray:
    """(D, D, D, 3) float32 smoothed uniform RGB albedo."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed + 7919)
    a = rng.uniform(lo, hi, size=(D, D, D, 3))
    for ch in range(3):
        a[..., ch] = gaussian_filter(a[..., ch], sigma=smooth, mode="nearest")
    return np.clip(a, lo, hi).astype(np.float32)


@dataclass
class VolumeConfig:
    name: str
    grid: int
    res: int
    spp: int
    max_depth: int
    steps: int
    lr: float = 0.02
    albedo: float | None = 0.8  # None -> RGB albedo grid
    spp_ref: int = 256
    init: float = 1.0
    seed: int = 0
    clamp: tuple = (0.0, 250.0)
    blobs: int = 8  # Gaussian blobs of the density
    extra: dict = field(default_factory=dict)

    @property
    def spp_grad(self) -> int:
        return self.spp

    def paths_per_step(self) -> int:
        return self.res * self.res * (self.spp + self.spp_grad)


CONFIGS = {
    # 32^3 density, constant albedo, 128^2, spp 4, depth 16, 50 Adam steps
    "cfg1": VolumeConfig("cfg1", grid=32, res=128, spp=4, max_depth=16, steps=50),
    # 64^3 density + 64^3 RGB albedo, 512^2, spp 16, depth 64, 200 steps
    "cfg2": VolumeConfig("cfg2", grid=64, res=512, spp=16, max_depth=64, steps=200, albedo=None),
    # profiling cases: the cfg2 medium at 128^2 and 256^2 (one launch = 262 144
    # and 1 048 576 paths)
    "cfg2s": VolumeConfig("cfg2s", grid=64, res=128, spp=16, max_depth=64, steps=200, albedo=None),
    "cfg2m": VolumeConfig("cfg2m", grid=64, res=256, spp=16, max_depth=64, steps=200, albedo=None),
    # a sparse medium for the majorant supergrid: one Gaussian blob in a 128^3
    # grid (mostly empty space), 512^2, spp 16, depth 64
    "sparse128": VolumeConfig("sparse128", grid=128, res=512, spp=16, max_depth=64, steps=200, blobs=1),
}


def medium_dict(density, albedo, box=None) -> dict:
    """``heterogeneous`` medium dictionary; ``box`` (a ``core.BoxTransform``)
    is the grids' ``to_world``."""
    grid = {"type": "gridvolume", "data": density}
    if box is not None:
        grid["to_world"] = box
    m = {
        "type": "heterogeneous",
        "sigma_t": grid,
        "scale": 1.0,
        "phase": {"type": "isotropic"},
    }
    if albedo is None or np.isscalar(albedo) or np.asarray(albedo).ndim <= 1:
        m["albedo"] = albedo if albedo is not None else 0.8
    else:
        m["albedo"] = {"type": "gridvolume", "data": albedo}
        if box is not None:
            m["albedo"]["to_world"] = box
    return m


def scene_dict(density, albedo, res: int, two_state: bool = True, spp: int = 4, box=None, views=None,
               height: int | None = None) -> dict:
    """Scene dictionary for ``load_dict`` (reference layout: a cube 'object'
    whose interior is a (two-state) medium, experiments.py:72-95).

    ``box``: the medium's ``to_world`` (``core.T.translate(t).scale(s)``).
    ``views``: (origin, target, up) triples of a ``batch`` sensor of
    len(views) sub-sensors, each with a res x height film
    (experiments.py:28-50); default one perspective sensor."""
    med = medium_dict(density, albedo, box)
    interior = {"type": "twostatemedium", "old": med, "new": med, "incoming": med} if two_state else med
    h = res if height is None else int(height)
    sampler = {"type": "independent", "sample_count": spp}
    if views is None:
        sensor = {
            "type": "perspective",
            "fov": 45.0,
            "to_world": look_at(CAMERA_ORIGIN, CAMERA_TARGET, CAMERA_UP),
            "film": {"type": "hdrfilm", "width": res, "height": h, "rfilter": {"type": "box"}},
            "sampler": sampler,
        }
    else:
        sensor = {
            "type": "batch",
            "film": {"type": "hdrfilm", "width": res * len(views), "height": h, "rfilter": {"type": "box"}},
            "sampler": sampler,
        }
        for i, (o, t, u) in enumerate(views):
            sensor[f"sensor_{i:02d}"] = {"type": "perspective", "fov": 45.0, "to_world": look_at(o, t, u)}
    obj = {"type": "cube", "bsdf": {"type": "null"}, "interior": interior}
    if box is not None:
        obj["to_world"] = box
    return {
        "type": "scene",
        "sensor": sensor,
        "emitter": {"type": "constant", "radiance": 1.0},
        "object": obj,
    }


def orbit_views(box, n: int, distance: float = 2.0, height: float = 0.0, phase: float = 0.1):
    """n look-at views on a circle around the box centre (the batch sensors
    of experiments.py:44-50,157-164)."""
    lo = np.array(box.box_min if box is not None else (0.0, 0.0, 0.0), np.float64)
    size = np.array(box.box_size if box is not None else (1.0, 1.0, 1.0), np.float64)
    c = lo + 0.5 * size
    views = []
    for i in range(n):
        th = 2 * np.pi / n * i + phase
        o = (c[0] + distance * np.cos(th), c[1] + height, c[2] + distance * np.sin(th))
        views.append((o, tuple(c), (0.0, 1.0, 0.0)))
    return views


def config_grids(cfg: VolumeConfig, seed: int | None = None):
    """True density / albedo of a configuration (albedo is a float when constant)."""
    s = cfg.seed if seed is None else seed
    dens = blob_density(cfg.grid, s, n_blobs=cfg.blobs)
    alb = cfg.albedo if cfg.albedo is not None else albedo_grid(cfg.grid, s)
    return dens, alb


def majorant_factor_for(density_res) -> int:
    """Supergrid factor of utils.adjust_majorant_res_factor (utils.py:27-43):
    8, reduced until the smallest side has at least 4 supergrid cells; 0 (no
    supergrid) when even factor 2 does not."""
    f = 8
    min_side = int(min(density_res[:3]))
    while f > 1 and min_side // f < 4:
        f -= 1
    return f if f > 1 else 0


DENSITY_KEY = "object.interior_medium.sigma_t.data"
ALBEDO_KEY = "object.interior_medium.albedo.data"

# ------------------------------------------------------------ surface scenes
TEXTURE_KEY = "plane.bsdf.reflectance.data"
SURFACE_CAMERA = ((0.0, 2.5, 4.5), (0.0, 0.3, 0.0), (0.0, 1.0, 0.0))


def value_noise(res: int, seed: int, octaves: int = 4, base: int = 4) -> np.ndarray:
    """(res, res, 3) float32 RGB value noise in [0.05, 0.95]: `octaves`
    lattices of seeded uniform values (base, 2 base, ... cells per side),
    smoothstep-interpolated, amplitudes halving per octave."""
    rng = np.random.default_rng(seed)
    x = (np.arange(res) + 0.5) / res
    out = np.zeros((res, res, 3))
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = base * 2**o
        lat = rng.uniform(0.0, 1.0, size=(cells + 1, cells + 1, 3))
        g = x * cells
        i0 = np.floor(g).astype(int)
        f = g - i0
        s = f * f * (3.0 - 2.0 * f)
        v = (lat[i0][:, i0] * (1 - s)[:, None, None] * (1 - s)[None, :, None]
             + lat[i0 + 1][:, i0] * s[:, None, None] * (1 - s)[None, :, None]
             + lat[i0][:, i0 + 1] * (1 - s)[:, None, None] * s[None, :, None]
             + lat[i0 + 1][:, i0 + 1] * s[:, None, None] * s[None, :, None])
        out += amp * v
        total += amp
        amp *= 0.5
    out /= total
    return (0.05 + 0.9 * out).astype(np.float32)


def surface_spheres(seed: int, n: int = 3):
    """n spheres with radii U[0.2, 0.5] resting on the ground, seeded colours."""
    rng = np.random.default_rng(seed + 104729)
    out = []
    for _ in range(n):
        r = float(rng.uniform(0.2, 0.5))
        cx, cz = rng.uniform(-1.2, 1.2, size=2)
        alb = tuple(float(v) for v in rng.uniform(0.3, 0.9, size=3))
        out.append(((float(cx), r, float(cz)), r, alb))
    return out


def surface_scene_dict(texture, res: int, seed: int = 0, spp: int = 8, light_radiance: float = 15.0) -> dict:
    """Ground plane ([-2, 2]^2 at y = 0, two-state textured diffuse), three
    diffuse spheres and one 1 x 1 area light at y = 3 (config 3)."""
    tex_bsdf = {"type": "diffuse", "reflectance": {"type": "bitmap", "data": texture}}
    d = {
        "type": "scene",
        "sensor": {
            "type": "perspective",
            "fov": 45.0,
            "to_world": look_at(*SURFACE_CAMERA),
            "film": {"type": "hdrfilm", "width": res, "height": res, "rfilter": {"type": "box"}},
            "sampler": {"type": "independent", "sample_count": spp},
        },
        "plane": {"type": "rectangle", "ground": True, "half_size": 2.0,
                  "bsdf": {"type": "twostate", "old": tex_bsdf, "new": tex_bsdf, "incoming": tex_bsdf}},
        "light": {"type": "rectangle", "center": (0.0, 3.0, 0.0), "half_size": (0.5, 0.5),
                  "emitter": {"type": "area", "radiance": light_radiance}},
    }
    for k, (c, r, alb) in enumerate(surface_spheres(seed)):
        sb = {"type": "diffuse", "reflectance": alb}
        d[f"sphere{k}"] = {"type": "sphere", "center": c, "radius": r,
                           "bsdf": {"type": "twostate", "old": sb, "new": sb, "incoming": sb}}
    return d


@dataclass
class SurfaceConfig:
    name: str
    res: int
    tex_res: int
    spp: int
    max_depth: int
    rr_depth: int
    steps: int
    lr: float = 0.02
    init: float = 0.5
    seed: int = 0

    @property
    def spp_grad(self) -> int:
        return self.spp

    def paths_per_step(self) -> int:
        return self.res * self.res * (self.spp + self.spp_grad)


SURFACE_CONFIGS = {
    # 1024^2, 512^2 RGB texture from 0.5 grey, spp 8, depth 8, 300 steps
    "cfg3": SurfaceConfig("cfg3", res=1024, tex_res=512, spp=8, max_depth=8, rr_depth=5, steps=300),
}
