"""Host-side behaviour of the plugin mirror (no GPU): registry, the
reference's error behaviour, seeds, parameter traversal and state rotation."""
import numpy as np
import pytest
import torch

import recursive_control_variates_gb300 as rcv
from recursive_control_variates_gb300 import scenes


def cpu_scene(two_state=True, albedo=0.8, D=4):
    dens = scenes.blob_density(D, 0)
    d = scenes.scene_dict(dens, albedo, res=8, two_state=two_state)
    return rcv.load_dict(d, device="cpu")


def test_plugin_names_registered():
    from recursive_control_variates_gb300.core import _KINDS

    for name in ("cv", "meta", "twostateprbvolpath", "twostateprb", "prbvolpath", "volpathsimple"):
        assert _KINDS[name] == "integrator"
    assert _KINDS["twostatemedium"] == "medium"


def test_volpathsimple_options():
    """Switches of plugins/volpathsimple.py:33-48 (all on by default) and its
    use as the `adjoint_integrator` of `cv` (experiments.py:131,245,364)."""
    v = rcv.load_dict({"type": "volpathsimple"})
    f = v.flags()
    assert (f.use_nee, f.use_drt, f.use_drt_subsampling, f.use_drt_mis) == (1, 1, 1, 1)
    v = rcv.load_dict({"type": "volpathsimple", "use_drt_mis": False, "use_nee": False, "max_depth": 12})
    f = v.flags()
    assert (f.use_nee, f.use_drt, f.use_drt_subsampling, f.use_drt_mis) == (0, 1, 1, 0)
    assert v.max_depth == 12 and "use_drt_mis = False" in v.to_string()
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath"},
                           "adjoint_integrator": {"type": "volpathsimple"}})
    assert type(integ.adjoint_integrator).__name__ == "VolpathSimpleIntegrator"
    assert v._checked_medium(cpu_scene(two_state=False)) is not None  # a plain medium is accepted


def test_cv_requires_two_state_integrator():
    with pytest.raises(ValueError, match="twostate"):
        rcv.load_dict({"type": "cv", "integrator": {"type": "prbvolpath"}})
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath", "max_depth": 16, "rr_depth": 16}})
    assert integ.warmup == 1 and integ.beta1 == 0.9 and integ.beta2 == 0.999
    assert integ.adjoint_integrator is integ.integrator
    assert integ.integrator.max_depth == 16


def test_meta_options():
    with pytest.raises(ValueError):
        rcv.load_dict({"type": "meta", "method": "cv_ps", "denoise": True, "integrator": {"type": "twostateprbvolpath"}})
    with pytest.raises(ValueError):
        rcv.load_dict({"type": "meta", "method": "bogus", "integrator": {"type": "twostateprbvolpath"}})
    m = rcv.load_dict({"type": "meta", "method": "cv_ps", "pre_update": True, "integrator": {"type": "twostateprbvolpath"}})
    assert m.pre_update and m.method == "cv_ps"


def test_check_scene_requires_two_state_medium():
    integ = rcv.load_dict({"type": "twostateprbvolpath"})
    with pytest.raises(RuntimeError, match="No TwoStateMedium"):
        integ.check_scene(cpu_scene(two_state=False))
    integ.check_scene(cpu_scene(two_state=True))


def test_unknown_plugin_and_unsupported_options():
    with pytest.raises(ValueError):
        rcv.load_dict({"type": "nope"})
    with pytest.raises(ValueError):
        rcv.load_dict({"type": "constant", "radiance": 2.0})
    dens = scenes.blob_density(4, 0)
    bad = scenes.medium_dict(dens, 0.8)
    bad["majorant_resolution_factor"] = -1
    with pytest.raises(ValueError):
        rcv.load_dict(bad, device="cpu")


@pytest.mark.parametrize("kind", ["twostateprbvolpath", "prbvolpath", "twostateprb"])
def test_adjoint_options(kind):
    """The adjoint choice of the volume and surface integrators reaches the C
    options: the event tape by default, the replay on request; unknown names
    and tape sizes outside [0, 16] are rejected."""
    from recursive_control_variates_gb300 import _lib
    o = rcv.load_dict({"type": kind}).options()
    assert o.adjoint == _lib.ADJOINT_TAPE and o.tape_events_per_path == 0
    o = rcv.load_dict({"type": kind, "adjoint": "replay", "tape_events_per_path": 4}).options()
    assert o.adjoint == _lib.ADJOINT_REPLAY and o.tape_events_per_path == 4
    with pytest.raises(ValueError):
        rcv.load_dict({"type": kind, "adjoint": "none"})
    with pytest.raises(ValueError):
        rcv.load_dict({"type": kind, "tape_events_per_path": 17})
    with pytest.raises(ValueError):
        rcv.load_dict({"type": kind, "tape_events_per_path": -1})


def test_majorant_resolution_factor():
    """`majorant_resolution_factor` (experiments.py:70,187,306) is accepted on the
    heterogeneous media; the two-state medium reports and sets the factor of
    its states (plugins/twostatemedium.py:171-178)."""
    dens = scenes.blob_density(16, 0)
    m = scenes.medium_dict(dens, 0.8)
    m["majorant_resolution_factor"] = 8
    med = rcv.load_dict(m, device="cpu")
    assert med.majorant_resolution_factor() == 8 and med.c_struct().majorant_factor == 8
    scene = cpu_scene()
    tm = scene.named_shapes()["object"].interior_medium()
    assert tm.majorant_resolution_factor() == 0
    tm.set_majorant_resolution_factor(4)
    assert tm.majorant_resolution_factor() == 4 and tm.c_struct().majorant_factor == 4
    assert tm.old.majorant_factor == tm.incoming.majorant_factor == 4
    with pytest.raises(ValueError):
        tm.set_majorant_resolution_factor(-2)


def test_seed_rules():
    assert rcv.default_seed_grad(5) == rcv.sample_tea_32(5, 1)[0]
    scene = cpu_scene()
    integ = rcv.load_dict({"type": "twostateprbvolpath"})
    with pytest.raises(Exception, match="different"):
        rcv.render(scene, None, integ, seed=3, seed_grad=3, spp=4)


def test_traverse_keys_and_rotation():
    scene = cpu_scene(albedo=scenes.albedo_grid(4, 0))
    params = rcv.traverse(scene)
    assert set(params.keys()) == {scenes.DENSITY_KEY, scenes.ALBEDO_KEY}
    med = scene.named_shapes()["object"].interior_medium()
    first = med.new.density.clone()
    a = torch.full_like(first, 2.0)
    b = torch.full_like(first, 3.0)
    params[scenes.DENSITY_KEY] = a
    params.update()
    assert torch.equal(med.old.density, first) and torch.equal(med.new.density, a)
    params[scenes.DENSITY_KEY] = b
    params.update()
    assert torch.equal(med.old.density, a) and torch.equal(med.new.density, b)
    assert torch.equal(med.incoming.density, b)
    with pytest.raises(ValueError):
        params[scenes.DENSITY_KEY] = torch.zeros(2, 2, 2, 3)  # wrong channel count


def test_upsample_resizes_all_states():
    """utils.upsample (utils.py:177-192): nearest-neighbour doubling of the
    optimised grid (Dr.Jit's tensor upsample), supergrid factor re-chosen,
    integrator reset; the next params.update gives old = new = incoming the
    new resolution."""
    scene = cpu_scene(D=4)
    params = rcv.traverse(scene)
    opt = rcv.ad.Adam(lr=0.1, device="cpu")
    g = torch.arange(64, dtype=torch.float32).reshape(4, 4, 4, 1)
    opt[scenes.DENSITY_KEY] = g
    params.update(opt)
    integ = rcv.load_dict({"type": "cv", "integrator": {"type": "twostateprbvolpath"}})
    integ.init_buffers()
    assert integ.init
    rcv.utils.upsample(scene, {"variables": {scenes.DENSITY_KEY: {}}, "use_majorant_supergrid": True}, opt, integ)
    up = opt[scenes.DENSITY_KEY]
    assert tuple(up.shape) == (8, 8, 8, 1) and not integ.init
    assert torch.equal(up[::2, ::2, ::2], g) and torch.equal(up[1::2, 1::2, 1::2], g)
    params.update(opt)
    med = scene.named_shapes()["object"].interior_medium()
    for st in (med.old, med.new, med.incoming):
        assert tuple(st.density.shape) == (8, 8, 8, 1) and torch.equal(st.density, up.detach())
    assert med.majorant_resolution_factor() == 2  # largest f with 8 // f >= 4
    assert rcv.utils.upsample_steps(2000, [0.04, 0.16, 0.36, 0.64]) == [80, 320, 720, 1280]
    with pytest.raises(ValueError):
        rcv.utils.upsample_grid(torch.zeros(3, 3, 1), shape=(4, 4, 1))


def test_box_transforms_and_batch_sensor(tmp_path):
    """T.scale / T.translate compose like Mitsuba's transforms; the medium
    box reaches the C struct; a `batch` sensor fills one frame per
    sub-sensor with the sub-film aspect (experiments.py:28-50,285)."""
    from recursive_control_variates_gb300.core import T

    tw = T.translate([0.5, -1.0, 2.0]).scale([6.5, 7.5, 10])
    assert tw.box_min == (0.5, -1.0, 2.0) and tw.box_size == (6.5, 7.5, 10.0)
    tw2 = T.scale([2, 2, 2]).translate([1, 0, 0])  # x -> 2 (x + t)
    assert tw2.box_min == (2.0, 0.0, 0.0)
    with pytest.raises(ValueError):
        T.scale([1, -1, 1])
    dens = scenes.blob_density(4, 0)
    med = {"type": "heterogeneous", "sigma_t": {"type": "gridvolume", "data": dens, "to_world": tw},
           "albedo": 0.8, "scale": 2.0}
    obj = tmp_path / "cube_unit.obj"
    obj.write_text("".join(f"v {x} {y} {z}\n" for x in (0, 1) for y in (0, 1) for z in (0, 1)) + "f 1 2 3\n")
    sensors = {f"sensor_{i:02d}": {"type": "perspective", "fov": 45,
                                   "to_world": T.look_at(origin=[3 * i, 1, 5], target=[3, 4, 7], up=[0, 1, 0])}
               for i in range(4)}
    batch = {"type": "batch", "film": {"type": "hdrfilm", "width": 4 * 16, "height": 12}, **sensors}
    scene = rcv.load_dict({"type": "scene", "sensor": batch, "emitter": {"type": "constant"},
                           "object": {"type": "obj", "filename": str(obj), "bsdf": {"type": "null"},
                                      "to_world": tw, "interior": med}}, device="cpu")
    m = scene.named_shapes()["object"].interior_medium().c_struct()
    assert tuple(m.box_min) == (0.5, -1.0, 2.0) and tuple(m.box_size) == (6.5, 7.5, 10.0)
    s = scene.sensors()[0].c_struct()
    assert (s.width, s.height, s.count) == (64, 12, 4)
    assert tuple(s.origin) == (0.0, 1.0, 5.0) and tuple(s.more[2].origin) == (9.0, 1.0, 5.0)
    # right / up scaled with the sub-film aspect 16:12
    r, u = np.array(s.right), np.array(s.up)
    assert np.isclose(np.linalg.norm(u) / np.linalg.norm(r), 12 / 16, rtol=1e-6)
    with pytest.raises(ValueError):  # shape and grid disagree on to_world
        rcv.load_dict({"type": "obj", "filename": str(obj), "to_world": T.scale([1, 2, 1]),
                       "interior": med}, device="cpu")
    bad = tmp_path / "not_a_cube.obj"
    bad.write_text("v 0 0 0\nv 2 1 1\n")
    with pytest.raises(ValueError):
        rcv.load_dict({"type": "obj", "filename": str(bad)}, device="cpu")
    with pytest.raises(ValueError):  # 64 px do not split into 3 sensors
        rcv.load_dict({"type": "batch", "film": {"type": "hdrfilm", "width": 64, "height": 12},
                       **{k: sensors[k] for k in list(sensors)[:3]}})


def _zips_half_exr(img):
    """A ZIPS-compressed OpenEXR file with half channels B, G, R, made with
    the published steps: byte interleave, predictor, zlib."""
    import struct
    import zlib

    from recursive_control_variates_gb300 import io

    h, w, _ = img.shape
    chlist = b"".join(n + b"\0" + struct.pack("<i4xii", 1, 1, 1) for n in (b"B", b"G", b"R")) + b"\0"
    box = struct.pack("<4i", 0, 0, w - 1, h - 1)
    header = struct.pack("<ii", 20000630, 2)
    header += io._attr("channels", "chlist", chlist)
    header += io._attr("compression", "compression", bytes([2]))
    header += io._attr("dataWindow", "box2i", box)
    header += io._attr("displayWindow", "box2i", box)
    header += io._attr("lineOrder", "lineOrder", bytes([0]))
    header += b"\0"
    planes = img[:, :, [2, 1, 0]].transpose(0, 2, 1).astype("<f2")  # per line: B, G, R
    chunks, offsets = b"", []
    base = len(header) + 8 * h
    for y in range(h):
        t = np.frombuffer(planes[y].tobytes(), np.uint8)
        inter = np.concatenate([t[0::2], t[1::2]]).astype(np.int64)
        pred = inter.copy()
        pred[1:] = (inter[1:] - inter[:-1] + 128) & 0xFF
        comp = zlib.compress(pred.astype(np.uint8).tobytes())
        if len(comp) >= t.size:  # the format stores such chunks uncompressed
            comp = t.tobytes()
        offsets.append(base + len(chunks))
        chunks += struct.pack("<ii", y, len(comp)) + comp
    return header + struct.pack(f"<{h}Q", *offsets) + chunks


def test_vol_and_exr_files(tmp_path):
    """Mitsuba .vol grids and OpenEXR images: round trips, a ZIPS EXR with
    half channels, and a gridvolume loaded from a file with its bbox."""
    from recursive_control_variates_gb300 import io

    g = np.random.default_rng(0).random((3, 4, 5, 3)).astype(np.float32)
    io.write_vol(tmp_path / "a.vol", g, (0, 0, 0), (1.0, 1.2, 1.5))
    v = io.read_vol(tmp_path / "a.vol")
    assert np.array_equal(v.data, g) and np.allclose(v.bbox_max, (1.0, 1.2, 1.5))
    img = np.random.default_rng(1).random((7, 9, 3)).astype(np.float32)
    io.write_exr(tmp_path / "a.exr", img)
    assert np.array_equal(io.read_exr(tmp_path / "a.exr"), img)
    # smooth rows compress, random rows are stored raw
    smooth = np.broadcast_to(np.linspace(0, 1, 40, dtype=np.float32)[None, :, None], (6, 40, 3)).copy()
    for im in (img, smooth):
        (tmp_path / "z.exr").write_bytes(_zips_half_exr(im))
        np.testing.assert_array_equal(io.read_exr(tmp_path / "z.exr"), im.astype(np.float16).astype(np.float32))
    io.write_vol(tmp_path / "d.vol", scenes.blob_density(4, 0), (1, 2, 3), (2, 4, 6))
    gv = rcv.load_dict({"type": "gridvolume", "filename": str(tmp_path / "d.vol"), "use_grid_bbox": True},
                       device="cpu")
    assert gv.to_world.box_min == (1.0, 2.0, 3.0) and gv.to_world.box_size == (1.0, 2.0, 3.0)
    assert np.array_equal(np.asarray(gv.raw), scenes.blob_density(4, 0))
