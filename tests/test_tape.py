"""The tape adjoint of the volume tracer (kTape radiance pass + rcv_tape.cu)
against the checkpoint replay and the CPU oracle.

Both adjoints scatter the same per-event values (path replay
backpropagation: null collisions, real scattering events, shadow-walk steps,
plugins/twostatevolpath.py:141-479); only the order of the float atomic
additions differs, so the two gradients agree within 1e-6 relative L2 and
each agrees with the oracle's double-precision sums within 2e-5.  A tape
too small for the events (tape_events_per_path) loses paths, which the
replay then traces whole: the gradient must not change."""
import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import scenes

from test_gpu_volume import make_scene, oracle_scene

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def grads_of(cuda, scene, gimg, seed, spp, max_depth=8, **props):
    integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": max_depth, "rr_depth": max_depth,
                           "overlap_adjoint": False, **props})
    g = integ.render_backward(scene, rcv.traverse(scene), torch.from_numpy(gimg).to(cuda), 0, seed=seed, spp=spp)
    torch.cuda.synchronize()
    out = {k: v.detach().cpu().numpy().copy() for k, v in g.items()}
    return out


@pytest.mark.parametrize("albedo_grid", [False, True])
@pytest.mark.parametrize("per_path", [0, 4, 1])
def test_tape_matches_replay_and_oracle(cuda, oracle, albedo_grid, per_path):
    """per_path 0: the full tape (16 slots per path); 4 and 1: most paths
    lose events and are replayed whole."""
    scene, med, grids = make_scene(cuda, albedo_grid=albedo_grid, res=32)
    gimg = np.random.default_rng(9).normal(0, 1, (32, 32, 3)).astype(np.float32)
    tape = grads_of(cuda, scene, gimg, 77, 4, adjoint="tape", tape_events_per_path=per_path)
    replay = grads_of(cuda, scene, gimg, 77, 4, adjoint="replay")
    od, oa = oracle.backward(oracle_scene(oracle, scene, grids, 8, albedo_grid), seed=77, spp=4, grad_img=gimg)
    gd = tape[scenes.DENSITY_KEY][..., 0]
    assert np.linalg.norm(od) > 0
    assert rel_l2(gd, replay[scenes.DENSITY_KEY][..., 0]) <= 1e-6
    assert rel_l2(gd, od) <= 2e-5, rel_l2(gd, od)
    if albedo_grid:
        ga = tape[scenes.ALBEDO_KEY]
        assert np.linalg.norm(oa) > 0
        assert rel_l2(ga, replay[scenes.ALBEDO_KEY]) <= 1e-6
        assert rel_l2(ga, oa) <= 2e-5, rel_l2(ga, oa)


@pytest.mark.parametrize("max_depth", [1, 3, 64])
def test_tape_depth_limits(cuda, oracle, max_depth):
    """Paths that end at the depth limit (no event for the last real
    collision) and deep paths that walk their last steps cooperatively."""
    scene, med, grids = make_scene(cuda, res=24, max_depth=max_depth)
    gimg = np.random.default_rng(max_depth).normal(0, 1, (24, 24, 3)).astype(np.float32)
    tape = grads_of(cuda, scene, gimg, 5, 8, max_depth=max_depth)
    od, _ = oracle.backward(oracle_scene(oracle, scene, grids, max_depth, False), seed=5, spp=8, grad_img=gimg)
    replay = grads_of(cuda, scene, gimg, 5, 8, max_depth=max_depth, adjoint="replay")
    gd = tape[scenes.DENSITY_KEY][..., 0]
    assert rel_l2(gd, replay[scenes.DENSITY_KEY][..., 0]) <= 1e-6
    assert rel_l2(gd, od) <= 2e-5, rel_l2(gd, od)


@pytest.mark.parametrize("factor,per_path", [(4, 0), (8, 0), (4, 3)])
def test_tape_under_supergrid(cuda, oracle, factor, per_path):
    """With a majorant supergrid the tape keeps each event's majorant (the
    DDA cell's) beside it: the gradient equals the replay's and the
    oracle's (per_path 3: most paths replayed whole)."""
    scene, med, grids = make_scene(cuda, albedo_grid=True, D=24, res=32)
    med.set_majorant_resolution_factor(factor)
    gimg = np.random.default_rng(factor).normal(0, 1, (32, 32, 3)).astype(np.float32)
    tape = grads_of(cuda, scene, gimg, 31, 4, tape_events_per_path=per_path)
    replay = grads_of(cuda, scene, gimg, 31, 4, adjoint="replay")
    od, oa = oracle.backward(oracle_scene(oracle, scene, grids, 8, True, factor), seed=31, spp=4, grad_img=gimg)
    gd = tape[scenes.DENSITY_KEY][..., 0]
    assert rel_l2(gd, replay[scenes.DENSITY_KEY][..., 0]) <= 1e-6
    assert rel_l2(gd, od) <= 2e-5, rel_l2(gd, od)
    assert rel_l2(tape[scenes.ALBEDO_KEY], oa) <= 2e-5


def test_tape_counters_match_replay(cuda):
    """The tape's gradient scatter counts the same events as the replay."""
    scene, med, grids = make_scene(cuda, res=24, albedo_grid=True)
    gimg = np.random.default_rng(2).normal(0, 1, (24, 24, 3)).astype(np.float32)
    counts = {}
    for mode in ("tape", "replay"):
        integ = rcv.load_dict({"type": "twostateprbvolpath", "max_depth": 8, "rr_depth": 8, "adjoint": mode,
                               "count_events": True, "overlap_adjoint": False})
        integ.counters(cuda).zero_()
        integ.render_backward(scene, rcv.traverse(scene), torch.from_numpy(gimg).to(cuda), 0, seed=1, spp=4)
        c = integ.counters(cuda).cpu().numpy()
        counts[mode] = (int(c[4]), int(c[5]))
    assert counts["tape"] == counts["replay"] and counts["tape"][0] > 0
