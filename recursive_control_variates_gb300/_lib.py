"""ctypes binding of librcv (include/rcv.h).

The library is the only compute path of this package: if it cannot be built or
loaded, every call that needs it raises instead of falling back to anything.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import _build

RCV_OK = 0
RCV_ERR_INVALID = -1
RCV_ERR_CUDA = -2
RCV_ERR_UNSUPPORTED = -3

COUNTER_PATHS = 0
COUNTER_LOOKUPS = 1
COUNTER_NEE_LOOKUPS = 2
COUNTER_SCATTERS = 3
COUNTER_GRAD_EVENTS = 4
COUNTER_ALBEDO_EVENTS = 5
COUNTER_COUNT = 8

LOSS_L2 = 0
LOSS_L1 = 1

f3 = C.c_float * 3
i3 = C.c_int32 * 3


MAX_SENSORS = 16


class CameraFrame(C.Structure):
    _fields_ = [("origin", f3), ("forward", f3), ("right", f3), ("up", f3)]


class Sensor(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("origin", f3),
        ("forward", f3),
        ("right", f3),
        ("up", f3),
        ("count", C.c_int32),
        ("pad", C.c_int32),
        ("more", CameraFrame * (MAX_SENSORS - 1)),
    ]


class Medium(C.Structure):
    _fields_ = [
        ("dims", i3),
        ("scale", C.c_float),
        ("density_old", C.c_void_p),
        ("density_new", C.c_void_p),
        ("albedo_old", C.c_void_p),
        ("albedo_new", C.c_void_p),
        ("albedo_value", f3),
        ("majorant_factor", C.c_int32),
        ("workspace", C.c_void_p),
        ("box_min", f3),
        ("box_size", f3),
        ("albedo_dims", i3),
        ("pad", C.c_int32),
    ]


class VolpathOptions(C.Structure):
    _fields_ = [
        ("max_depth", C.c_int32),
        ("rr_depth", C.c_int32),
        ("hide_emitters", C.c_int32),
        ("batch", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("defer", C.c_int32),
        ("order", C.c_int32),
        ("count_events", C.c_int32),
        ("envmap", C.c_void_p),  # const rcv_envmap* or NULL (constant environment)
        ("adjoint", C.c_int32),  # ADJOINT_TAPE / ADJOINT_REPLAY
        ("tape_events_per_path", C.c_int32),  # 1..16, 0 = 16
        ("separate_tracers", C.c_int32),  # 1: two-state and adjoint radiance passes as two launches
    ]


class Envmap(C.Structure):
    _fields_ = [
        ("width", C.c_int32),
        ("height", C.c_int32),
        ("scale", C.c_float),
        ("pad", C.c_int32),
        ("texels", C.c_void_p),
        ("workspace", C.c_void_p),
    ]


class VpsFlags(C.Structure):
    _fields_ = [
        ("use_nee", C.c_int32),
        ("use_drt", C.c_int32),
        ("use_drt_subsampling", C.c_int32),
        ("use_drt_mis", C.c_int32),
    ]


ORDER_COST = 0
ORDER_ROW_MAJOR = 1
ORDER_LONGEST_FIRST = 2
ORDERS = {"cost": ORDER_COST, "row_major": ORDER_ROW_MAJOR, "longest_first": ORDER_LONGEST_FIRST}


MODE_TWOSTATE = 0
MODE_SINGLE = 1
MODE_ADJOINT = 2

ADJOINT_TAPE = 0
ADJOINT_REPLAY = 1
ADJOINTS = {"tape": ADJOINT_TAPE, "replay": ADJOINT_REPLAY}


class SphereDesc(C.Structure):
    _fields_ = [("center", f3), ("radius", C.c_float), ("albedo", f3)]


MAX_SPHERES = 8


class SurfaceScene(C.Structure):
    _fields_ = [
        ("plane_half", C.c_float),
        ("tex_width", C.c_int32),
        ("tex_height", C.c_int32),
        ("tex_old", C.c_void_p),
        ("tex_new", C.c_void_p),
        ("num_spheres", C.c_int32),
        ("spheres", SphereDesc * MAX_SPHERES),
        ("light_center", f3),
        ("light_half", C.c_float * 2),
        ("light_radiance", f3),
        ("workspace", C.c_void_p),
    ]


class CvState(C.Structure):
    _fields_ = [(name, C.c_void_p) for name in ("img", "w_s", "v_n", "mean_x", "mean_y", "var_x", "var_y", "cov")]


class BatchJob(C.Structure):
    _fields_ = [
        ("sensor", Sensor),
        ("dims", i3),
        ("scale", C.c_float),
        ("albedo_value", f3),
        ("spp", C.c_int32),
        ("spp_grad", C.c_int32),
        ("max_depth", C.c_int32),
        ("rr_depth", C.c_int32),
        ("hide_emitters", C.c_int32),
        ("seed_base", C.c_uint32),
        ("warmup", C.c_int32),
        ("pre_update", C.c_int32),
        ("cv_beta1", C.c_float),
        ("cv_beta2", C.c_float),
        ("cv_table1", C.c_void_p),
        ("cv_table2", C.c_void_p),
        ("cv_table1_len", C.c_int32),
        ("cv_table2_len", C.c_int32),
        ("loss", C.c_int32),
        ("lr", C.c_float),
        ("adam_beta1", C.c_float),
        ("adam_beta2", C.c_float),
        ("adam_eps", C.c_float),
        ("density_lo", C.c_float),
        ("density_hi", C.c_float),
        ("albedo_lo", C.c_float),
        ("albedo_hi", C.c_float),
        ("adam_table", C.c_void_p),
        ("adam_table_len", C.c_int32),
        ("majorant_factor", C.c_int32),
        ("box_min", f3),
        ("box_size", f3),
        ("density", C.c_void_p * 2),
        ("albedo", C.c_void_p * 2),
        ("density_m", C.c_void_p),
        ("density_v", C.c_void_p),
        ("albedo_m", C.c_void_p),
        ("albedo_v", C.c_void_p),
        ("target", C.c_void_p),
        ("cv", CvState),
        ("img_old", C.c_void_p),
        ("img_new", C.c_void_p),
        ("workspace", C.c_void_p),
    ]


class BatchJobStatus(C.Structure):
    _fields_ = [
        ("it", C.c_int32),
        ("welford_count", C.c_int32),
        ("adam_t", C.c_int32),
        ("pad", C.c_int32),
        ("loss_sum", C.c_double),
        ("loss", C.c_float),
        ("pad1", C.c_float),
    ]


vp = C.c_void_p
P = C.POINTER

# name -> (restype, argtypes); every symbol of include/rcv.h
SIGNATURES = {
    "rcv_last_error": (C.c_char_p, []),
    "rcv_kernel_launches": (C.c_uint64, []),
    "rcv_device_info": (C.c_int, [P(C.c_int32), P(C.c_int32), P(C.c_int32)]),
    "rcv_struct_size": (C.c_uint64, [C.c_char_p]),
    "rcv_sample_tea_32": (None, [C.c_uint32, C.c_uint32, P(C.c_uint32)]),
    "rcv_medium_workspace_bytes": (C.c_uint64, [P(C.c_int32), C.c_int32, C.c_int32]),
    "rcv_medium_workspace_bytes_for": (C.c_uint64, [P(Medium)]),
    "rcv_medium_prepare": (C.c_int, [P(Medium), vp]),
    "rcv_envmap_workspace_bytes": (C.c_uint64, [C.c_int32, C.c_int32]),
    "rcv_envmap_prepare": (C.c_int, [P(Envmap), vp]),
    "rcv_render_workspace_bytes": (C.c_uint64, [C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "rcv_render_twostates_volume": (
        C.c_int,
        [P(Medium), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp, vp, vp],
    ),
    "rcv_render_volume": (
        C.c_int, [P(Medium), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp, vp]
    ),
    "rcv_render_volume_noalloc": (
        C.c_int, [P(Medium), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp]
    ),
    "rcv_render_backward_volume": (
        C.c_int,
        [P(Medium), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp, vp, vp, vp],
    ),
    "rcv_render_forward_volume": (
        C.c_int,
        [P(Medium), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp, vp, vp, vp],
    ),
    "rcv_render_adjoint_radiance": (
        C.c_int, [P(Medium), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp]
    ),
    "rcv_render_twostates_volume_and_adjoint_radiance": (
        C.c_int,
        [P(Medium), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp, C.c_uint32, C.c_int32, vp, vp,
         vp],
    ),
    "rcv_render_backward_replay": (
        C.c_int,
        [P(Medium), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp, vp, vp, vp],
    ),
    "rcv_volpathsimple_workspace_bytes": (C.c_uint64, [C.c_int32, C.c_int32, C.c_int32]),
    "rcv_render_volpathsimple": (
        C.c_int, [P(Medium), P(Sensor), P(VolpathOptions), P(VpsFlags), C.c_uint32, C.c_int32, vp, vp, vp]
    ),
    "rcv_render_backward_volpathsimple": (
        C.c_int,
        [P(Medium), P(Sensor), P(VolpathOptions), P(VpsFlags), C.c_uint32, C.c_int32, vp, vp, vp, vp],
    ),
    "rcv_surface_workspace_bytes": (C.c_uint64, [C.c_int32, C.c_int32]),
    "rcv_surface_prepare": (C.c_int, [P(SurfaceScene), vp]),
    "rcv_render_twostates_surface": (
        C.c_int, [P(SurfaceScene), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp, vp, vp]
    ),
    "rcv_render_surface": (
        C.c_int, [P(SurfaceScene), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp, vp]
    ),
    "rcv_render_backward_surface": (
        C.c_int, [P(SurfaceScene), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp, vp, vp]
    ),
    "rcv_render_forward_surface": (
        C.c_int, [P(SurfaceScene), P(Sensor), P(VolpathOptions), C.c_uint32, C.c_int32, vp, vp, vp, vp, vp]
    ),
    "rcv_cv_step": (
        C.c_int,
        [P(CvState), C.c_int64, vp, vp, C.c_int32, C.c_int32, P(C.c_int32), C.c_float, C.c_float, C.c_int32, vp],
    ),
    "rcv_statistics_get": (C.c_int, [P(CvState), C.c_int64, C.c_int32, C.c_float, vp, vp, vp, vp]),
    "rcv_statistics_update": (C.c_int, [P(CvState), C.c_int64, vp, vp, P(C.c_int32), C.c_float, C.c_float, vp]),
    "rcv_clamp": (C.c_int, [vp, C.c_int64, C.c_float, C.c_float, vp]),
    "rcv_cv_table_len": (C.c_int64, [C.c_float]),
    "rcv_cv_table_fill": (C.c_int, [C.c_float, vp, C.c_int64]),
    "rcv_adam_table_len": (C.c_int64, [C.c_float, C.c_float]),
    "rcv_adam_table_fill": (C.c_int, [C.c_float, C.c_float, vp, C.c_int64]),
    "rcv_batch_job_workspace_bytes": (C.c_uint64, [P(BatchJob)]),
    "rcv_batch_job_init": (C.c_int, [P(BatchJob), vp]),
    "rcv_batch_workspace_bytes": (C.c_uint64, [P(BatchJob), C.c_int32]),
    "rcv_batch_create": (C.c_int, [P(BatchJob), C.c_int32, P(VolpathOptions), vp, C.c_uint64, P(vp), vp]),
    "rcv_batch_step": (C.c_int, [vp, C.c_int32, vp]),
    "rcv_batch_counters": (vp, [vp]),
    "rcv_batch_kernels_per_step": (C.c_int32, [vp]),
    "rcv_batch_destroy": (C.c_int, [vp]),
    "rcv_welford_update": (C.c_int, [vp, vp, C.c_int64, vp, P(C.c_int32), C.c_float, C.c_float, vp]),
    "rcv_welford_get": (C.c_int, [vp, C.c_int64, C.c_int32, C.c_float, vp, vp]),
    "rcv_loss_workspace_bytes": (C.c_uint64, [C.c_int64]),
    "rcv_loss": (C.c_int, [C.c_int32, vp, vp, C.c_int64, vp, vp, vp, vp]),
    "rcv_adam_step": (
        C.c_int,
        [vp, vp, vp, vp, C.c_int64, C.c_int32, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
         C.c_int32, vp],
    ),
}

_lock = threading.Lock()
_lib: C.CDLL | None = None


def library_path() -> Path:
    return _build.lib_path()


# ctypes mirrors of the public structs, checked against the library at load
STRUCTS = {
    "rcv_camera_frame": CameraFrame,
    "rcv_sensor": Sensor,
    "rcv_medium": Medium,
    "rcv_volpath_options": VolpathOptions,
    "rcv_sphere": SphereDesc,
    "rcv_surface_scene": SurfaceScene,
    "rcv_cv_state": CvState,
    "rcv_batch_job": BatchJob,
    "rcv_batch_job_status": BatchJobStatus,
    "rcv_volpathsimple_flags": VpsFlags,
    "rcv_envmap": Envmap,
}


def load() -> C.CDLL:
    """Loads librcv, building it first when the sources changed."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.build()
        lib = C.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        for cname, struct in STRUCTS.items():
            got, want = int(lib.rcv_struct_size(cname.encode())), C.sizeof(struct)
            if got != want:
                raise RuntimeError(f"librcv {cname} is {got} bytes, the binding's {want}: stale build")
        _lib = lib
        return lib


class RCVError(RuntimeError):
    pass


def check(rc: int, what: str = "") -> None:
    if rc == RCV_OK:
        return
    msg = load().rcv_last_error().decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if rc == RCV_ERR_INVALID:
        raise ValueError(text)
    raise RCVError(f"{text} (code {rc})")


def sample_tea_32(v0: int, v1: int) -> tuple[int, int]:
    out = (C.c_uint32 * 2)()
    load().rcv_sample_tea_32(C.c_uint32(v0 & 0xFFFFFFFF), C.c_uint32(v1 & 0xFFFFFFFF), out)
    return int(out[0]), int(out[1])
