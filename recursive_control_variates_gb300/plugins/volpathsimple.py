"""Simplified volumetric path tracer with differential ratio tracking
(``volpathsimple``, plugins/volpathsimple.py:23-778 of the reference).

The reference's grid experiments hand it to the ``cv`` / ``meta``
integrators as ``adjoint_integrator`` (experiments.py:131,245,364): the
primal images come from the two-state tracer, the gradients from this
integrator's adjoint.  Switches (plugins/volpathsimple.py:33-48):
``use_nee``, ``use_drt``, ``use_drt_subsampling``, ``use_drt_mis``, all on
by default.  ``render`` and ``render_backward`` run on the GPU through
librcv (rcv_render_volpathsimple / rcv_render_backward_volpathsimple).
"""
from __future__ import annotations

import ctypes as C

import torch

from .. import _lib, profiling
from ..utils import stream_handle
from .twostatevolpath import _SRGB_TO_XYZ, PRBVolpathIntegrator


class VolpathSimpleIntegrator(PRBVolpathIntegrator):
    """``volpathsimple``: delta tracking to real interactions, NEE towards the
    environment with MIS, and an adjoint with DRT for the in-scattering term."""

    def __init__(self, props):
        super().__init__(props)
        self.use_nee = bool(props.get("use_nee", True))
        self.use_drt = bool(props.get("use_drt", True))
        self.use_drt_subsampling = bool(props.get("use_drt_subsampling", True))
        self.use_drt_mis = bool(props.get("use_drt_mis", True))
        self._vps_scratch: dict[torch.device, torch.Tensor] = {}

    def render_forward(self, scene, params, sensor=0, seed: int = 0, spp: int = 0, tangents=None):
        """The reference's sample() has a primal and an adjoint branch only
        (plugins/volpathsimple.py:64): no forward mode."""
        raise NotImplementedError("volpathsimple has no forward mode (plugins/volpathsimple.py:64); "
                                  "use render_backward, or prbvolpath / twostateprbvolpath for forward mode")

    def prefetch_adjoint(self, scene, sensor=0, seed: int = 0, spp: int = 0):
        """The DRT adjoint is one launch per call: nothing to start ahead."""
        return None

    def flags(self) -> _lib.VpsFlags:
        f = _lib.VpsFlags()
        f.use_nee = int(self.use_nee)
        f.use_drt = int(self.use_drt)
        f.use_drt_subsampling = int(self.use_drt_subsampling)
        f.use_drt_mis = int(self.use_drt_mis)
        return f

    def _path_scratch(self, device, sensor, spp: int) -> int:
        device = torch.device(device)
        f = sensor.film()
        need = int(_lib.load().rcv_volpathsimple_workspace_bytes(f.width, f.height, spp)) + 256
        buf = self._vps_scratch.get(device)
        if buf is None or buf.numel() < need:
            buf = torch.empty(need, dtype=torch.uint8, device=device)
            self._vps_scratch[device] = buf
        return (buf.data_ptr() + 255) & ~255

    def render(self, scene, sensor=0, seed: int = 0, spp: int = 0, develop: bool = True, evaluate: bool = True):
        """Primal image of the current parameters
        (VolpathSimpleIntegrator.sample in primal mode, :53-327)."""
        medium = self._checked_medium(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        st = stream_handle(medium.device)
        m = medium.prepare(st)
        s = sensor.c_struct()
        o = self.options(scene)
        fl = self.flags()
        img = self._image(sensor, medium.device)
        with profiling.region("vps_primal", medium.device):
            _lib.check(
                _lib.load().rcv_render_volpathsimple(
                    C.byref(m), C.byref(s), C.byref(o), C.byref(fl), seed & 0xFFFFFFFF, spp, img.data_ptr(),
                    self._path_scratch(medium.device, sensor, spp), st,
                ),
                "rcv_render_volpathsimple",
            )
        return self._post(img)

    def render_backward(self, scene, params, grad_in: torch.Tensor, sensor=0, seed: int = 0, spp: int = 0):
        """Adjoint of the current parameters: ``{key: gradient}`` for the
        density (and albedo grid) keys present in ``params``."""
        medium = self._checked_medium(scene)
        sensor = self.sensor_of(scene, sensor)
        spp = self.resolve_spp(sensor, spp)
        if self.xyz:
            grad_in = grad_in @ _SRGB_TO_XYZ.to(grad_in.device)
        g = grad_in.detach().to(medium.device, torch.float32).contiguous()
        f = sensor.film()
        if tuple(g.shape) != (f.height, f.width, 3):
            raise ValueError(f"grad_in has shape {tuple(g.shape)}, expected {(f.height, f.width, 3)}")
        st = stream_handle(medium.device)
        m = medium.prepare(st)
        s = sensor.c_struct()
        o = self.options(scene)
        fl = self.flags()
        dx, dy, dz = medium.dims
        gd = torch.zeros((dz, dy, dx, 1), dtype=torch.float32, device=medium.device)
        ga = medium.albedo_grad_buffer()
        with profiling.region("vps_adjoint", medium.device):
            _lib.check(
                _lib.load().rcv_render_backward_volpathsimple(
                    C.byref(m), C.byref(s), C.byref(o), C.byref(fl), seed & 0xFFFFFFFF, spp, g.data_ptr(),
                    gd.data_ptr(), ga.data_ptr() if ga is not None else None, st,
                ),
                "rcv_render_backward_volpathsimple",
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

    def to_string(self):
        return (
            f"VolpathSimpleIntegrator[max_depth = {self.max_depth}, use_nee = {self.use_nee}, "
            f"use_drt = {self.use_drt}, use_drt_subsampling = {self.use_drt_subsampling}, "
            f"use_drt_mis = {self.use_drt_mis}]"
        )

