"""Scene construction (gg_scene_build) against an independent restatement of
loadSceneConfig / init_granular_system (main.cu:123-188, 746-1173); no GPU."""
import json
import math
import os

import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
SCENES = os.path.join(HERE, "golden", "scenes")
from oracle.ref_cuda_build import REF_ROOT  # noqa: E402

REF_SCENES = os.path.join(REF_ROOT, "scenes")  # skipped where the checkout is absent
F = np.float32


def _minstd_uniform(count, a, b):
    """std::default_random_engine (minstd_rand0, seed 1) through
    uniform_real_distribution<float>(a, b), libstdc++'s generate_canonical."""
    out = np.empty(count, np.float32)
    x = 1
    span = F(F(b) - F(a))
    r = F(2147483646.0)
    for k in range(count):
        x = (x * 16807) % 2147483647
        c = F(F(x - 1) / r)
        if c >= F(1):
            c = np.nextafter(F(1), F(0))
        out[k] = F(F(c * span) + F(a))
    return out


def restate(path):
    j = json.load(open(path))
    v = lambda k: np.array([j[k]["x"], j[k]["y"], j[k]["z"]], np.float32)
    space, box = v("space_size"), v("box_size")
    s = F(j["init_spacing"])
    L = F(j["cell_length"])
    pt, bt = v("particle_translation"), v("boundary_translation")
    cs = [int(math.ceil(F(space[k] / L))) for k in range(3)]
    parts = []
    i = 0
    while F(i) < box[0]:
        jj = 0
        while F(jj) < box[1]:
            k = 0
            while F(k) < box[2]:
                parts.append(np.array([F(0.27) + F(s * F(jj)), F(0.13) + F(s * F(i)), F(0.17) + F(s * F(k))],
                                      np.float32) + pt)
                k += 1
            jj += 1
        i += 1
    parts = np.array(parts, np.float32).reshape(-1, 3)
    draws = _minstd_uniform(parts.shape[0] * 25 * 3, -0.01, 0.01).reshape(-1, 3)
    offs = draws[:, ::-1]  # z takes the first draw (right-to-left argument evaluation)
    ups = (np.repeat(parts, 25, 0) + offs).astype(np.float32)
    c = [2 * x for x in cs]
    den = np.array([c[0] - 1, c[1] - 1, c[2] - 1], np.float32)
    walls = []
    w = lambda a, b_, cc: walls.append(F(0.99) * (np.array([a, b_, cc], np.float32) / den * space) + F(0.005) * space)
    sc = j["scene"]
    anim = []
    if sc in (1, 5, 4, 2, 3):
        back = sc != 4
        for a in range(c[0]):
            for b_ in range(c[1]):
                w(a, b_, 0)
                if back:
                    w(a, b_, c[2] - 1)
    top = sc in (0, 1, 5)
    if sc in (0, 1, 5, 4, 2, 3):
        for a in range(c[0]):
            for b_ in range(c[2] - 2):
                w(a, 0, b_ + 1)
                if top:
                    w(a, c[1] - 1, b_ + 1)
    if sc in (1, 5, 4, 2, 3):
        right = sc != 4
        for a in range(c[1] - 2):
            for b_ in range(c[2] - 2):
                w(0, a + 1, b_ + 1)
                if right:
                    w(c[0] - 1, a + 1, b_ + 1)
    walls = np.array(walls, np.float32).reshape(-1, 3)
    if sc in (0, 1, 4, 5):
        walls = (walls + bt).astype(np.float32)
    anim = np.zeros(walls.shape[0], np.int32)
    if sc == 3 and j.get("obj_file"):
        pts = np.loadtxt(os.path.join(os.path.dirname(path), j["obj_file"]), dtype=np.float32).reshape(-1, 3)
        cen = np.zeros(3, np.float32)
        for p in pts:
            cen = (cen + p).astype(np.float32)
        cen = (cen / F(len(pts))).astype(np.float32)
        ang = F(90.0 * math.pi / 180.0)
        ct, st = F(math.cos(ang)), F(math.sin(ang))
        extra = []
        for p in pts:
            q = (p - cen).astype(np.float32)
            ny = F(F(q[1] * ct) - F(q[2] * st))
            nz = F(F(q[1] * st) + F(q[2] * ct))
            extra.append(((np.array([q[0], ny, nz], np.float32) + cen) + np.array([1.25, 0.3, 1.5], np.float32)))
        walls = np.concatenate([walls, np.array(extra, np.float32)])
        anim = np.concatenate([anim, np.ones(len(extra), np.int32)])
    return parts, ups, walls, anim, cs


@pytest.mark.parametrize("name", ["box_small.json", "corner_small.json", "funnel_small.json"])
def test_scene_build_matches_restatement(name):
    path = os.path.join(SCENES, name)
    sc = gg.scene_build(path, base_dir=SCENES)
    parts, ups, walls, anim, cs = restate(path)
    assert np.array_equal(sc["particles"], parts)
    assert np.array_equal(sc["upsampled"], ups)
    assert np.array_equal(sc["boundary"], walls)
    assert np.array_equal(sc["boundary_animated"], anim)
    assert tuple(sc["cell_size"]) == tuple(cs)


def test_scene_errors_are_reported(tmp_path):
    with pytest.raises(gg.GranularError) as e:
        gg.scene_build(str(tmp_path / "missing.json"))
    assert e.value.status == abi.GG_ERR_IO
    bad = tmp_path / "bad.json"
    bad.write_text('{"space_size": {"x": 1, "y": 1, "z": 1}, "dt": ')
    with pytest.raises(gg.GranularError) as e:
        gg.scene_build(str(bad))
    assert e.value.status == abi.GG_ERR_PARSE
    j = json.load(open(os.path.join(SCENES, "box_small.json")))
    del j["cell_length"]
    miss = tmp_path / "miss.json"
    miss.write_text(json.dumps(j))
    with pytest.raises(gg.GranularError) as e:
        gg.scene_build(str(miss))
    assert e.value.status == abi.GG_ERR_PARSE and "cell_length" in str(e.value)


@pytest.mark.skipif(not os.path.isdir(REF_SCENES), reason="reference scene files not present")
def test_reference_scene_files_load():
    expect = {"box.json": 100000, "corner.json": 100000, "excavator.json": 100000, "funnel.json": 60840,
              "piling.json": 8, "box_opening_no.json": 8, "box_opening_up.json": 8}
    for name, n in expect.items():
        sc = gg.scene_build(os.path.join(REF_SCENES, name), base_dir=os.path.dirname(REF_SCENES))
        assert len(sc["particles"]) == n, name
        assert len(sc["upsampled"]) == 25 * n, name
    box = gg.scene_build(os.path.join(REF_SCENES, "box.json"))
    assert tuple(box["cell_size"]) == (50, 45, 45)
    assert len(box["boundary"]) == 2 * 100 * 90 + 2 * 100 * 88 + 2 * 88 * 88
    exc = gg.scene_build(os.path.join(REF_SCENES, "excavator.json"), base_dir=os.path.dirname(REF_SCENES))
    assert exc["is_move_boundary"] == 1 and int(exc["boundary_animated"].sum()) == 13045
