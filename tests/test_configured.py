"""Configured mode: the contact model the benchmark configurations describe
(Coulomb friction with static and kinetic coefficients, restitution 0,
analytic walls, split children that claim their cell), which the
reference's compiled-in constants cannot express.

Checked against the CPU oracle bit for bit (math mode 1) through every
sweep kernel, and physically: friction holds a block on a 30-degree plane
to a slight creep when mu_static > tan 30 and lets it slide when
mu_kinetic is small, and the
column collapse runs the configuration's 200 frames (800 substeps) with no
NaN, no particle through the floor and exact mass units.
"""
import math

import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import abi, workloads
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _configured_box(lists=True):
    desc = workloads.box_drop(n_side=12, substeps=4, iters=5, adaptive=1, upsample_per=2)
    rng = np.random.default_rng(4)
    desc["masses"] = rng.choice(np.array([1.0, 1.0, 2.0, 3.0], np.float32), desc["n_particles"])
    planes = workloads.box_planes(desc["space_size"]) + [((-0.5, math.sqrt(3) / 2, 0.0), 0.2)]
    workloads.configure(desc["params"], 0.5, 0.4, planes)
    desc["params"].mass_ledger = 1
    desc["params"].math_mode = 1
    if not lists:
        desc["params"].nlist_skin = 0.0
    return desc


@pytest.mark.parametrize("variant,lists", [(0, True), (0, False), (1, True)])
def test_configured_mode_matches_oracle(variant, lists):
    desc = _configured_box(lists)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), masses=desc["masses"], device=0)
    s.set_tuning(sweep_variant=variant)
    o = orc.OracleSystem(desc, fp64=False)
    split = 0
    for k in range(1, 50):
        s.step(1)
        o.step(1)
        assert s.size() == o.size(), f"substep {k}: {s.size()} vs {o.size()} particles"
        for f in (gg.FIELD_POS, gg.FIELD_VEL, gg.FIELD_MASS_UNITS, gg.FIELD_NUM_CONSTRAINTS, gg.FIELD_REMOVE):
            a, b = s.read(f), o.read(f)
            assert np.array_equal(a, b), f"substep {k}: field {f} differs at {np.nonzero((a != b).reshape(len(a), -1).any(1))[0][:5]}"
        split += s.stats()["split_last"]
    assert s.stats()["total_mass_units"] == round(float(np.sum(desc["masses"], dtype=np.float64)) * abi.UNITS_PER_MASS)
    assert split > 0, "the scene must split (children claim their cells)"
    s.close()
    o.close()


def _block_on_ramp(mu_s, mu_k, substeps=60):
    """A 6 x 4 x 6 block resting on a 30-degree analytic plane (no other
    wall), friction mu_s / mu_k; returns the block's centre-of-mass
    displacement along the slope after `substeps` of 1/240 s."""
    r = 0.01
    th = math.radians(30.0)
    t = np.array([math.cos(th), math.sin(th), 0.0])
    nrm = np.array([-math.sin(th), math.cos(th), 0.0])
    p0 = np.array([0.5, 0.35, 0.5])
    pts = []
    for i in range(6):
        for j in range(4):
            for k in range(6):
                pts.append(p0 + (i - 2.5) * 2 * r * t + (r * 1.001 + j * 2 * r) * nrm + np.array([0, 0, (k - 2.5) * 2 * r]))
    p = np.array(pts, np.float32)
    desc = workloads.box_drop(n_side=2, substeps=4, iters=5, adaptive=0, upsample_per=0)
    desc.update(particles=p, n_particles=p.shape[0], boundary=np.zeros((0, 3), np.float32), n_boundary=0,
                skip_initial_step=1)
    workloads.configure(desc["params"], mu_s, mu_k, [(nrm, float(nrm @ p0))])
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    c0 = s.read(gg.FIELD_POS).astype(np.float64).mean(0)
    s.step(substeps)
    c1 = s.read(gg.FIELD_POS).astype(np.float64).mean(0)
    pen = float((s.read(gg.FIELD_POS).astype(np.float64) @ nrm - nrm @ p0).min())
    s.close()
    return float((c1 - c0) @ t), pen


def test_friction_holds_or_releases_a_block_on_a_30_degree_plane():
    # tan 30 = 0.577.  Without friction the block slides about
    # g sin 30 t^2 / 2 = 0.15 m in 0.25 s; mu 0.7 holds it to a creep of
    # about a tenth of that (Jacobi sweeps carry the block's weight down to
    # the bottom layer over several substeps, so the layers above shear a
    # little), mu 0.1 lets it slide about half as far as without friction
    # (measured with the oracle: 0.156, 0.016, 0.080 m)
    free, pen_f = _block_on_ramp(0.0, 0.0)
    stick, pen_s = _block_on_ramp(0.7, 0.7)
    slide, pen_l = _block_on_ramp(0.1, 0.1)
    assert free < -0.12, free
    assert abs(stick) < 0.15 * abs(free), (stick, free)
    assert 0.35 * abs(free) < abs(slide) < 0.7 * abs(free), (slide, free)
    assert min(pen_f, pen_s, pen_l) > -0.002  # nobody sinks into the plane


def test_configured_column_runs_200_frames():
    # the column-collapse configuration's 200 frames (dt = 1/120 in 4
    # substeps) at a size a test finishes quickly
    desc = workloads.column_collapse(counts=(24, 48, 48), constants="configured", upsample_per=1)
    n0 = desc["n_particles"]
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    floor = 0.005 * desc["space_size"][1]
    for frame in range(200):
        s.step(4)
        if frame % 50 == 49:
            st = s.stats()
            assert st["nonfinite"] == 0, f"frame {frame}: NaN positions"
            assert st["total_mass_units"] == n0 * abi.UNITS_PER_MASS
            y = s.read(gg.FIELD_POS)[:, 1]
            assert float(y.min()) >= floor, f"frame {frame}: {int((y < floor).sum())} particles below the floor"
    st = s.stats()
    assert st["merged_total"] > 0 and st["split_total"] > 0, st
    assert int(st["error_word"]) == 0
    s.close()


def _run_configured(desc, frames, substeps_per_frame, checks=4):
    """Steps a configured scene through its frames; checks NaN, the floor,
    the box and the mass ledger a few times on the way.  Returns the stats
    and the particle-substeps per second of the run."""
    import time
    n0 = desc["n_particles"]
    units0 = int(round(float(np.sum(desc.get("masses", np.ones(n0)), dtype=np.float64)) * abi.UNITS_PER_MASS))
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    sp = np.asarray(desc["space_size"], np.float32)
    lo, hi = 0.005 * sp, 0.995 * sp
    every = max(1, frames // checks)
    work = 0
    t0 = time.perf_counter()
    for frame in range(frames):
        work += s.size() * substeps_per_frame
        s.step(substeps_per_frame)
        if frame % every == every - 1 or frame == frames - 1:
            st = s.stats()
            assert st["nonfinite"] == 0, f"frame {frame}: NaN positions"
            assert st["total_mass_units"] == units0, f"frame {frame}: mass units"
            p = s.read(gg.FIELD_POS)
            assert np.all(p >= lo) and np.all(p <= hi), \
                f"frame {frame}: {int(np.sum(np.any((p < lo) | (p > hi), 1)))} particles outside the box"
    s.synchronize()
    rate = work / (time.perf_counter() - t0)
    st = s.stats()
    s.close()
    return st, rate


def test_box_drop_configuration_300_frames():
    # 32^3 particles, r = 0.01, dt = 1/60 in 4 substeps, 3 Jacobi sweeps,
    # friction 0.5 / 0.4, restitution 0: 300 frames
    st, rate = _run_configured(workloads.box_drop(n_side=32, substeps=4, iters=3, configured=True), 300, 4)
    print(f"box drop 32^3: {rate / 1e6:.1f} M particle-substeps/s (with the checks)")
    assert int(st["error_word"]) == 0


def test_adaptive_pile_configuration_600_frames():
    # 262,144 particles (r = 0.005) onto the floor and the 30-degree ramp,
    # merge/split up to mass 8, 4 render points each, dt = 1/240: 600 frames
    st, rate = _run_configured(workloads.adaptive_pile(configured=True), 600, 1)
    print(f"adaptive pile 262k: {rate / 1e6:.1f} M particle-substeps/s (with the checks)")
    assert st["merged_total"] > 0 and int(st["error_word"]) == 0


def test_column_collapse_configuration_200_frames_at_full_size():
    # 8,388,608 particles (r = 0.002), 33,554,432 render points, dt = 1/120
    # in 4 substeps, 4 Jacobi sweeps, merge/split up to mass 8: 200 frames
    desc = workloads.column_collapse(counts=(128, 256, 256), constants="configured")
    assert desc["n_particles"] == 8_388_608
    st, rate = _run_configured(desc, 200, 4)
    print(f"column collapse 8.4M: {rate / 1e6:.1f} M particle-substeps/s (with the checks)")
    assert st["merged_total"] > 0 and st["split_total"] > 0 and int(st["error_word"]) == 0


def test_configured_frames_replay_as_a_graph():
    # a configured scene without merge/split needs no host round trip: a
    # frame of 4 substeps replays as one CUDA graph, bit-equal to stepping
    def make():
        desc = workloads.box_drop(n_side=12, substeps=4, iters=3, configured=True)
        return gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    a, b = make(), make()
    b.graph_capture(4)
    for _ in range(5):
        a.step(4)
        b.graph_launch()
    b.synchronize()
    assert np.array_equal(a.read(gg.FIELD_POS), b.read(gg.FIELD_POS))
    assert np.array_equal(a.read(gg.FIELD_VEL), b.read(gg.FIELD_VEL))
    assert b.stats()["steps"] == a.stats()["steps"]
    a.close()
    b.close()
