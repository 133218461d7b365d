"""GB300-native recursive-control-variate gradient step.

Drop-in for the hot path of rgl-epfl/recursive_control_variates: the plugin
names and parameters of the reference (``cv``, ``meta``,
``twostateprbvolpath``, ``twostatemedium``, ...), a ``load_dict`` /
``traverse`` / ``render`` / ``ad.Adam`` host API in PyTorch, and hand-written
sm_103a CUDA kernels behind the C ABI of include/rcv.h (librcv.so).
"""
from . import ad, plugins
from ._lib import RCVError
from ._lib import load as load_library
from .core import (
    Properties,
    SceneParameters,
    load_dict,
    look_at,
    register_bsdf,
    register_integrator,
    register_medium,
    traverse,
)
from .render import default_seed_grad, render
from .utils import clamp, l1_loss, l2_loss, sample_tea_32

__all__ = [
    "ad",
    "plugins",
    "RCVError",
    "load_library",
    "Properties",
    "SceneParameters",
    "load_dict",
    "look_at",
    "register_bsdf",
    "register_integrator",
    "register_medium",
    "traverse",
    "render",
    "default_seed_grad",
    "clamp",
    "l1_loss",
    "l2_loss",
    "sample_tea_32",
]
