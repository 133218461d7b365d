"""The allocation-free render entry point, for callers that cannot allocate
device memory (code where cudaMalloc is unavailable or forbidden, or a host
that owns a fixed memory pool and passes this library only inputs and
outputs).  Called through the C ABI, it must give exactly the image of the
regular entry point on calls in a row of different film sizes, spp and
pixel orders (its static scratch keeps the previous call's contents), and
reject requests larger than its scratch.

This file is collected last so that, if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import _lib, scenes
from recursive_control_variates_gb300.utils import stream_handle

pytestmark = pytest.mark.gpu


def _scene(device, res):
    dens = scenes.blob_density(32, 3)
    alb = scenes.albedo_grid(32, 3)
    scene = rcv.load_dict(scenes.scene_dict(dens, alb, res=res), device=device)
    return scene, scene.named_shapes()["object"].interior_medium()


def _render_both(lib, cuda, res, height, spp, seed, order):
    """One call of each entry point on the same inputs; the regular one gets
    a fresh caller workspace, so its pixel order starts from no history."""
    scene = rcv.load_dict(scenes.scene_dict(scenes.blob_density(32, 3), scenes.albedo_grid(32, 3), res=res,
                                            height=height), device=cuda)
    med = scene.named_shapes()["object"].interior_medium()
    st = stream_handle(cuda)
    m = med.prepare(st)
    s = scene.sensors()[0].c_struct()
    o = _lib.VolpathOptions()
    o.max_depth, o.rr_depth, o.order = 16, 16, order
    nbytes = int(lib.rcv_render_workspace_bytes(res, height, spp, _lib.MODE_SINGLE))
    scratch = torch.zeros(nbytes + 256, dtype=torch.uint8, device=cuda)
    ws = (scratch.data_ptr() + 255) & ~255
    ref = torch.empty((height, res, 3), device=cuda)
    out = torch.full((height, res, 3), -1.0, device=cuda)
    _lib.check(lib.rcv_render_volume(C.byref(m), C.byref(s), C.byref(o), seed, spp, ref.data_ptr(), ws, None, st))
    _lib.check(lib.rcv_render_volume_noalloc(C.byref(m), C.byref(s), C.byref(o), seed, spp, out.data_ptr(), None,
                                             st))
    torch.cuda.synchronize()
    return out.cpu().numpy(), ref.cpu().numpy()


def test_noalloc_render_matches_regular_entry_point(cuda):
    """Calls in a row share the static scratch and find the previous call's
    pixel costs and order in it: a 64 x 64 call, a 96 x 48 call at another
    spp, a row-major call, and a 64 x 64 call again must each give the
    regular entry point's image bit for bit (stale costs only change the
    order in which pixels are handed out, never the result)."""
    lib = _lib.load()
    calls = [(64, 64, 16, 7, _lib.ORDER_COST), (96, 48, 8, 8, _lib.ORDER_COST),
             (64, 64, 16, 9, _lib.ORDER_ROW_MAJOR), (64, 64, 16, 10, _lib.ORDER_COST)]
    for res, height, spp, seed, order in calls:
        a, b = _render_both(lib, cuda, res, height, spp, seed, order)
        assert np.array_equal(a, b), f"{res}x{height} spp {spp}: max diff {np.abs(a - b).max()}"
        assert b.mean() > 0.05


def test_noalloc_render_rejects_oversized_requests(cuda):
    lib = _lib.load()
    scene, med = _scene(cuda, 1024)
    st = stream_handle(cuda)
    m = med.prepare(st)
    s = scene.sensors()[0].c_struct()
    o = _lib.VolpathOptions()
    o.max_depth, o.rr_depth = 16, 16
    out = torch.empty((1024, 1024, 3), device=cuda)
    rc = lib.rcv_render_volume_noalloc(C.byref(m), C.byref(s), C.byref(o), 1, 16, out.data_ptr(), None, st)
    assert rc == _lib.RCV_ERR_INVALID
    assert b"16 MiB" in lib.rcv_last_error()
