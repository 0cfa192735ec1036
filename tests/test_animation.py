"""The animated walls: AnimationState, updateAnimation and animateParticles
(main.cu:100-111, 1175-1277) against their restatement in oracle/.

The state machine is host code (CPU tests, bit for bit in float32); the
move runs on the GPU and is compared with the oracle's walls, and the
particles they push, substep by substep in math mode 1.
"""
import json
import os

import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import abi
from oracle import oracle as orc

F = np.float32
FIELDS = ("is_animating", "animation_time", "start_index", "num_particles", "translation_direction",
          "translation_speed", "translation_complete", "rotation_angle", "rotation_speed", "rotation_center")


def _as_dict(a):
    d = {}
    for k in FIELDS:
        v = getattr(a, k)
        d[k] = np.array(list(v), F) if k in ("translation_direction", "rotation_center") else v
    return d


def _same_state(a, d):
    for k in FIELDS:
        x, y = getattr(a, k), d[k]
        if k in ("translation_direction", "rotation_center"):
            assert np.array_equal(np.array(list(x), F), np.asarray(y, F)), k
        elif isinstance(x, float):
            assert F(x) == F(y), (k, x, y)
        else:
            assert int(x) == int(y), (k, x, y)


def _same_move(m, r):
    assert np.array_equal(np.array(list(m.translation), F), r["translation"])
    assert F(m.rotation) == r["rotation"]
    assert np.array_equal(np.array(list(m.center), F), r["center"])
    assert m.apply == r["apply"]


def test_defaults_are_the_reference_initialisers():
    a = gg.default_animation()
    assert a.is_animating == 0 and a.translation_complete == 0
    assert list(a.translation_direction) == [F(-0.1), 0.0, 0.0]
    assert a.translation_speed == 5.0 and a.rotation_speed == 90.0 and a.rotation_angle == 0.0


@pytest.mark.parametrize("dt", [1.0 / 60.0, 0.05, 0.3])
def test_state_machine_matches_restatement(dt):
    rng = np.random.default_rng(5)
    walls = rng.uniform(0.0, 1.0, (40, 3)).astype(F)
    a = gg.default_animation()
    a.is_animating, a.start_index, a.num_particles = 1, 7, 19
    r = _as_dict(a)
    phases = {"translate": 0, "rotate": 0}
    for frame in range(400):
        needs = gg.lib().gg_animation_needs_centroid(a, F(dt))
        m = gg.animation_advance(a, dt, walls if needs else None)
        mr = orc.animation_advance(r, dt, walls)
        _same_move(m, mr)
        _same_state(a, r)
        if m.apply and m.rotation == 0.0:
            phases["translate"] += 1
        if m.apply and m.rotation != 0.0:
            phases["rotate"] += 1
        if not a.is_animating:
            break
    # 2.5 s of translation, then 45 degrees at 90 degrees per second; the
    # frame that reaches 45 degrees moves nothing (the reference stops first)
    assert a.translation_complete == 1 and a.is_animating == 0 and a.rotation_angle >= 45.0
    assert phases["translate"] >= int(2.5 / dt) - 1
    cen = walls[7:26].astype(F).sum(0, dtype=F) / F(19)
    assert np.allclose(np.array(list(a.rotation_center)), cen, rtol=1e-6)
    # nothing happens once it has stopped
    m = gg.animation_advance(a, dt)
    assert m.apply == 0


def test_advance_needs_the_walls_when_the_translation_ends():
    a = gg.default_animation()
    a.is_animating, a.start_index, a.num_particles = 1, 0, 4
    a.animation_time = 2.49
    with pytest.raises(gg.GranularError):
        gg.animation_advance(a, 0.1)  # the centroid needs the wall positions
    assert a.animation_time == F(2.49) and a.translation_complete == 0  # the state is unchanged
    with pytest.raises(gg.GranularError):
        gg.animation_advance(a, 0.1, np.zeros((3, 3), F))  # the range lies outside the walls
    m = gg.animation_advance(a, 0.1, np.ones((4, 3), F))
    assert a.translation_complete == 1 and m.apply == 1 and m.rotation == F(-9.0)


def _excavator_scene(tmp_path):
    """Scene 2 (the excavator) with a 4 x 2 x 3 bucket of wall points: the
    bucket lands at +(2.5, 0, 0.5) and sweeps through a small pile."""
    g = np.stack(np.meshgrid(np.arange(4), np.arange(2), np.arange(3), indexing="ij"), -1).reshape(-1, 3)
    pts = (g * 0.02 + np.array([-0.2, 0.06, -0.28])).astype(F)
    np.savetxt(tmp_path / "bucket.txt", pts, fmt="%.4f")
    scene = {
        "space_size": {"x": 3.0, "y": 0.6, "z": 0.6}, "dt": 0.002, "gravity": {"x": 0.0, "y": -9.8, "z": 0.0},
        "sph_spacing": 0.02, "init_spacing": 0.021, "smoothing_radius": 0.04, "cell_length": 0.0404,
        "density": 238732.4146, "box_size": {"x": 6, "y": 4, "z": 6}, "scene": 2,
        "boundary_translation": {"x": 0.0, "y": 0.0, "z": 0.0},
        "particle_translation": {"x": 0.0, "y": 0.0, "z": 0.0},
        "obj_file": "bucket.txt", "is_adaptive": 0, "save_file": ""}
    path = tmp_path / "excavator_small.json"
    path.write_text(json.dumps(scene))
    return str(path), pts


def test_scene_animation_state(tmp_path):
    path, pts = _excavator_scene(tmp_path)
    sc = gg.scene_build(path, base_dir=str(tmp_path))
    a = gg.scene_animation(path, base_dir=str(tmp_path))
    nb = len(sc["boundary"])
    assert a.is_animating == 1 and a.num_particles == len(pts) and a.start_index == nb - len(pts)
    assert np.array_equal(sc["boundary_animated"][a.start_index:], np.ones(len(pts), np.int32))
    cen = np.zeros(3, F)
    for p in pts:
        cen = (cen + p).astype(F)
    cen = (cen / F(len(pts))).astype(F)
    assert np.array_equal(np.array(list(a.rotation_center), F), cen)  # before the bucket is placed
    fun = gg.scene_animation(os.path.join(os.path.dirname(__file__), "golden", "scenes", "funnel_small.json"),
                             base_dir=os.path.join(os.path.dirname(__file__), "golden", "scenes"))
    assert fun.is_animating == 1 and fun.num_particles == 4 and list(fun.rotation_center) == [0.0, 0.0, 0.0]
    box = gg.scene_animation(os.path.join(os.path.dirname(__file__), "golden", "scenes", "box_small.json"))
    assert box.is_animating == 0


@pytest.mark.gpu
def test_animated_walls_match_oracle(tmp_path):
    path, pts = _excavator_scene(tmp_path)
    sc = gg.scene_build(path, base_dir=str(tmp_path))
    prm = abi.default_params()
    prm.math_mode = 1
    s = gg.GranularSystem.from_scene(path, params=prm, base_dir=str(tmp_path))
    desc = dict(particles=sc["particles"], n_particles=len(sc["particles"]), boundary=sc["boundary"],
                n_boundary=len(sc["boundary"]), boundary_animated=sc["boundary_animated"],
                upsampled=sc["upsampled"], n_upsampled=len(sc["upsampled"]), space_size=sc["space_size"],
                cell_length=sc["cell_length"], dt=sc["dt"], gravity=sc["gravity"], cell_size=sc["cell_size"],
                density=sc["density"], upsampled_radius=sc["upsampled_radius"],
                is_move_boundary=sc["is_move_boundary"], is_adaptive=sc["is_adaptive"], skip_initial_step=0,
                device=0, max_particles=0, params=prm)
    assert sc["is_move_boundary"] == 1
    o = orc.OracleSystem(desc)
    a = gg.scene_animation(path, base_dir=str(tmp_path))
    r = _as_dict(a)
    frame_dt = 0.05
    rotated = 0
    for frame in range(70):
        walls_o = o.read(abi.FIELD_POS, abi.SET_BOUNDARY)
        assert np.array_equal(s.read(gg.FIELD_POS, gg.SET_BOUNDARY), walls_o), f"frame {frame}: walls"
        s.update_animation(a, frame_dt)
        mr = orc.animation_advance(r, frame_dt, walls_o)
        _same_state(a, r)
        if mr["apply"]:
            o.animate_walls(mr["translation"], mr["rotation"], mr["center"])
            rotated += mr["rotation"] != 0
        s.step(2)
        o.step(2)
        for f in (gg.FIELD_POS, gg.FIELD_VEL):
            x, y = s.read(f), o.read(f)
            assert np.array_equal(x, y), f"frame {frame}: field {f}"
        assert np.array_equal(s.read(gg.FIELD_IS_ANIMATED, gg.SET_BOUNDARY),
                              o.read(abi.FIELD_IS_ANIMATED, abi.SET_BOUNDARY))
    assert a.translation_complete == 1 and a.is_animating == 0 and rotated >= 9
    # the bucket moved: its flagged walls left their built positions
    anim = s.read(gg.FIELD_IS_ANIMATED, gg.SET_BOUNDARY) == 1
    bx = s.read(gg.FIELD_POS, gg.SET_BOUNDARY)[anim]
    assert bx[:, 0].max() < pts[:, 0].max() + 2.5 - 1.0
    s.close()
    o.close()
