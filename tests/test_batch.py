"""Batched scenes (needs a GPU): one system stepping independent scenes
side by side, per-scene friction and FP64 diagnostics, CUDA-graph replay."""
import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import batch as B, workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("law", ["coulomb", "cap"])
def test_batch_of_one_scene_equals_the_scene_alone(law):
    # Coulomb friction per scene (configured mode, the box faces as walls in
    # the scene's coordinates) or the reference's law with a cap per scene
    desc, info = B.batched_scenes(1, seed=3, lo=3000, hi=6000, law=law)
    b = B.Batch(desc, info)
    s = gg.GranularSystem(**workloads.system_kwargs(B.scene_desc(desc, info, 0)), device=0)
    b.system.step(30)
    s.step(30)
    assert np.array_equal(b.system.read(gg.FIELD_POS), s.read(gg.FIELD_POS))
    assert np.array_equal(b.system.read(gg.FIELD_VEL), s.read(gg.FIELD_VEL))
    b.close()
    s.close()


def test_scene_stats_match_separate_systems():
    n = 4
    desc, info = B.batched_scenes(n, seed=5, lo=2000, hi=9000)
    b = B.Batch(desc, info)
    alone = [gg.GranularSystem(**workloads.system_kwargs(B.scene_desc(desc, info, k)), device=0) for k in range(n)]
    b.system.step(10)
    for s in alone:
        s.step(10)
    st = b.scene_stats()
    for k, s in enumerate(alone):
        ref = s.stats()
        assert st[k, 0] == info["sizes"][k] == s.size()
        assert abs(st[k, 1] - ref["total_mass"]) <= 1e-9 * ref["total_mass"]
        com = np.array(ref["center_of_mass"]) + np.array([k * info["width"], 0, 0])
        assert np.abs(st[k, 6:9] - com).max() < 1e-5
        mom = np.array(ref["momentum"])
        assert np.abs(st[k, 2:5] - mom).max() <= 1e-3 * np.abs(mom).max() + 1e-6
        assert abs(st[k, 5] - ref["kinetic_energy"]) <= 1e-3 * ref["kinetic_energy"] + 1e-9
        s.close()
    b.close()


def test_friction_differs_per_scene():
    # the same block in two scenes with different friction caps: identical
    # until tangential corrections are capped, then not necessarily; the
    # scene table must at least reach the kernel (a cap of 0 changes the
    # wall corrections at once)
    desc, info = B.batched_scenes(2, seed=7, lo=3000, hi=3001)
    info["friction_cap"] = np.array([0.8, 0.0], np.float32)
    b = B.Batch(desc, info)
    b.system.step(60)
    st = b.scene_stats()
    assert st[0, 0] == st[1, 0]
    b.close()


def test_graph_replay_equals_stepping():
    desc, info = B.batched_scenes(3, seed=9, lo=3000, hi=8000)
    a = B.Batch(desc, info)
    c = B.Batch(desc, info)
    a.system.step(8)
    c.capture(4)
    c.launch()
    c.launch()
    assert np.array_equal(a.system.read(gg.FIELD_POS), c.system.read(gg.FIELD_POS))
    assert c.system.stats()["steps"] == 8
    a.close()
    c.close()


def test_graph_capture_refuses_host_round_trips():
    desc = workloads.box_drop(n_side=6, adaptive=1)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    from granular_gpu_gb300 import _check
    with pytest.raises(gg.GranularError):
        _check(gg.lib().gg_graph_capture(s._h, 2))
    s.close()


def test_autotune_restores_the_state_and_keeps_results():
    desc, info = B.batched_scenes(3, seed=11, lo=3000, hi=8000)
    a = B.Batch(desc, info)
    c = B.Batch(desc, info)
    a.system.step(4)
    c.system.step(4)
    t = c.autotune(2)
    assert t["trials"] == 10 and t["ms_tuned"] <= t["ms_default"]  # the defaults, then 9 other choices
    assert c.system.stats()["steps"] == a.system.stats()["steps"]
    assert np.array_equal(a.system.read(gg.FIELD_POS), c.system.read(gg.FIELD_POS))
    # launch shapes do not change results
    a.system.step(6)
    c.system.step(6)
    assert np.array_equal(a.system.read(gg.FIELD_POS), c.system.read(gg.FIELD_POS))
    a.close()
    c.close()


def test_coulomb_walls_and_coefficients_follow_each_scene():
    # two scenes, the second one slab over: the walls of gg_params.planes
    # hold each scene's particles inside its own box, and the per-scene
    # coefficients are the scenes' own (stepping each alone agrees)
    desc, info = B.batched_scenes(2, seed=8, lo=2000, hi=4000, law="coulomb")
    b = B.Batch(desc, info)
    alone = [gg.GranularSystem(**workloads.system_kwargs(B.scene_desc(desc, info, k)), device=0) for k in range(2)]
    b.system.step(10)
    for s in alone:
        s.step(10)
    st = b.scene_stats()
    p = b.system.read(gg.FIELD_POS)
    k = np.floor(p[:, 0] / info["width"]).astype(int)
    for j, s in enumerate(alone):
        q = p[k == j] - np.array([j * info["width"], 0, 0], np.float32)
        assert q.shape[0] == s.size() == st[j, 0]
        assert q.min() >= 0.005 and q.max() <= 0.995
        ref = s.stats()
        assert abs(st[j, 5] - ref["kinetic_energy"]) <= 1e-3 * ref["kinetic_energy"] + 1e-9
    b.close()
    for s in alone:
        s.close()
