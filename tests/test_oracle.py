"""The CPU oracle against the committed known-answer vectors (no GPU).

tests/golden/known_answers.json restates the reference's arithmetic for
tiny hand-checkable cases (tests/golden/make_golden.py).  Exact float32
agreement is expected except where libm's cbrtf/expf enter (1 ulp).
"""
import json
import os

import numpy as np
import pytest

from granular_gpu_gb300 import abi, workloads
from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))


def _desc(particles, boundary=None, upsampled=None, density=238732.4146, dt=0.002, g=(0.0, 0.0, 0.0),
          adaptive=0, params=None):
    p = np.asarray(particles, np.float32).reshape(-1, 3)
    b = np.zeros((0, 3), np.float32) if boundary is None else np.asarray(boundary, np.float32).reshape(-1, 3)
    u = None if upsampled is None else np.asarray(upsampled, np.float32).reshape(-1, 3)
    prm = params or abi.default_params()
    prm.upsample_enabled = 1 if u is not None else 0
    return dict(particles=p, n_particles=p.shape[0], boundary=b if len(b) else None, n_boundary=len(b),
                upsampled=u, n_upsampled=0 if u is None else u.shape[0], space_size=(1.0, 1.0, 1.0),
                cell_length=0.0404, dt=dt, gravity=g, cell_size=(25, 25, 25), density=density,
                upsampled_radius=0.005, is_move_boundary=0, is_adaptive=adaptive, skip_initial_step=1,
                device=0, max_particles=0, params=prm)


@pytest.mark.parametrize("fp64", [False, True])
def test_grid_known_answer(fp64):
    c = KA["grid"]
    k, sk, pm, cs = orc.grid_build(np.array(c["points"], np.float32), c["cell_size"], c["cell_length"], fp64=fp64)
    assert k.tolist() == c["keys"]
    assert sk.tolist() == c["sorted_keys"]
    assert pm.tolist() == c["perm"]
    assert cs.tolist() == c["cell_start"]


def test_pair_contact_known_answer():
    c = KA["pair"]
    o = orc.OracleSystem(_desc([c["x0"], c["x1"]], density=c["density"], dt=c["dt"]))
    o.step(1)
    pos = o.read(abi.FIELD_POS)
    assert np.allclose(pos, np.array(c["pos"], np.float32), rtol=0, atol=2e-7)
    assert np.allclose(o.read(abi.FIELD_VEL), np.array(c["vel"], np.float32), rtol=1e-4, atol=1e-4)
    assert o.read(abi.FIELD_CONTACTS).tolist() == c["contacts"]
    assert o.read(abi.FIELD_NUM_CONSTRAINTS).tolist() == c["num_constraints"]
    # momentum of the pair is conserved by the symmetric correction
    assert abs(float(o.read(abi.FIELD_VEL)[:, 0].sum())) < 1e-5


def test_wall_contact_known_answer():
    c = KA["wall"]
    o = orc.OracleSystem(_desc([c["x"]], boundary=[c["boundary"]], density=c["density"]))
    o.step(1)
    pos = o.read(abi.FIELD_POS)[0]
    assert np.allclose(pos, np.array(c["pos"], np.float32), atol=2e-7)
    sep = float(np.linalg.norm(pos.astype(np.float64) - np.array(c["boundary"])))
    assert sep == pytest.approx(0.02, abs=1e-6)


def test_final_velocity_damping_known_answer():
    c = KA["damping"]
    for case in c["cases"]:
        o = orc.OracleSystem(_desc([[0.3, 0.5, 0.5]], dt=c["dt"]))
        o.write(abi.FIELD_VEL, [[case["v0"], 0.0, 0.0]])
        o.step(1)
        assert o.read(abi.FIELD_POS)[0, 0] == np.float32(case["x"])
        assert o.read(abi.FIELD_VEL)[0, 0] == pytest.approx(case["velocity"], rel=2e-7, abs=1e-9)


def test_upsample_known_answer():
    c = KA["upsample"]
    o = orc.OracleSystem(_desc([c["particle"]], upsampled=[c["point"]]))
    o.step(1)
    assert np.allclose(o.read(abi.FIELD_VEL, abi.SET_UPSAMPLED)[0], c["vel"], rtol=1e-6, atol=1e-9)
    assert np.allclose(o.read(abi.FIELD_POS, abi.SET_UPSAMPLED)[0], c["pos"], rtol=0, atol=1e-7)


def test_fp32_restatement_tracks_fp64_transcription():
    desc = workloads.box_drop(n_side=8, substeps=4, iters=3)
    a = orc.OracleSystem(desc, fp64=False)
    b = orc.OracleSystem(desc, fp64=True)
    for _ in range(3):
        a.step(1)
        b.step(1)
    assert a.size() == b.size()
    err = np.abs(a.read(abi.FIELD_POS).astype(np.float64) - b.read(abi.FIELD_POS)).max()
    # FP32 rounding flips borderline contact decisions, so the two drift
    # apart by a fraction of an overlap; a loose sanity bound only
    assert err < 1e-3 * workloads.REF_RADIUS


def test_ledger_conserves_units_exactly():
    desc = workloads.box_drop(n_side=14, substeps=4, iters=5, adaptive=1)
    desc["params"].mass_ledger = 1
    desc["params"].max_mass = 8.0
    o = orc.OracleSystem(desc)
    total = desc["n_particles"] * abi.UNITS_PER_MASS
    merged = 0
    for _ in range(60):
        o.step(1)
        merged += o.merged_last()
        assert int(o.read(abi.FIELD_MASS_UNITS).astype(np.int64).sum()) == total
    assert merged > 0
    # masses are the units scaled exactly
    assert np.array_equal(o.read(abi.FIELD_MASS),
                          (o.read(abi.FIELD_MASS_UNITS).astype(np.float64) / abi.UNITS_PER_MASS).astype(np.float32))


def test_float_masses_drift_like_the_reference():
    # blending mass/40 forty times in FP32 (Solver.cu:669-671) does not
    # conserve the total exactly; the ledger above does
    desc = workloads.box_drop(n_side=14, substeps=4, iters=5, adaptive=1)
    o = orc.OracleSystem(desc)
    for _ in range(60):
        o.step(1)
    total = float(o.read(abi.FIELD_MASS).astype(np.float64).sum())
    assert abs(total - desc["n_particles"]) < 1e-3


def test_particle_stats_csv(tmp_path):
    desc = workloads.box_drop(n_side=6, substeps=4, iters=3, adaptive=1)
    o = orc.OracleSystem(desc)
    o.step(2)
    path = tmp_path / "stats.csv"
    o.save_particle_stats(str(path))
    lines = path.read_text().strip().splitlines()
    assert lines[0] == "Frame,MergedParticles,SplitParticles,TotalParticles"
    assert len(lines) == 1 + 3  # constructor step + 2 steps


def test_color_dots_known_answers():
    # generate_dots_CUDA (VBO.hpp:9-71) read as written
    p = np.arange(12, dtype=np.float32).reshape(4, 3)
    d, c = orc.color_dots(p, mass=[0, 1, 2.5, 4], mode=2)
    assert np.array_equal(d, p)
    assert np.isinf(c[0, 0]) and c[0, 1] == np.float32(214 / 255) and c[0, 2] == np.float32(160 / 255)
    assert np.array_equal(c[1:], np.array([[0, 0, 1], [0.5, 0, 0.5], [1, 0, 0]], np.float32))
    _, c = orc.color_dots(p, surface=[0, 1, 2, 1], mode=0)
    assert np.array_equal(c[:, 0], np.array([0, 0.34, 0, 0.34], np.float32))
    _, c = orc.color_dots(p, sdist=[0, 5, 100, np.nan], mode=1)
    assert np.array_equal(c, np.array([[0.34, 0.46, 0.7], [1, 0, 0], [0, 0, 0], [1, 0, 0]], np.float32))


def _ramp_block_slide(mu):
    """The oracle's configured mode: a 6 x 4 x 6 block on a 30-degree
    analytic plane, friction mu / mu; displacement along the slope after
    60 substeps of 1/240 s, and the deepest centre below the plane."""
    import math
    r = 0.01
    th = math.radians(30.0)
    t = np.array([math.cos(th), math.sin(th), 0.0])
    nrm = np.array([-math.sin(th), math.cos(th), 0.0])
    p0 = np.array([0.5, 0.35, 0.5])
    pts = [p0 + (i - 2.5) * 2 * r * t + (r * 1.001 + j * 2 * r) * nrm + np.array([0, 0, (k - 2.5) * 2 * r])
           for i in range(6) for j in range(4) for k in range(6)]
    p = np.array(pts, np.float32)
    desc = workloads.box_drop(n_side=2, substeps=4, iters=5, adaptive=0, upsample_per=0)
    desc.update(particles=p, n_particles=p.shape[0], boundary=np.zeros((0, 3), np.float32), n_boundary=0,
                skip_initial_step=1)
    workloads.configure(desc["params"], mu, mu, [(nrm, float(nrm @ p0))])
    o = orc.OracleSystem(desc, fp64=False)
    c0 = o.read(abi.FIELD_POS).astype(np.float64).mean(0)
    o.step(60)
    x = o.read(abi.FIELD_POS).astype(np.float64)
    o.close()
    return float((x.mean(0) - c0) @ t), float((x @ nrm - nrm @ p0).min())


def test_configured_friction_on_a_ramp():
    # the configured mode's Coulomb law in the oracle (the GPU kernels match
    # it bit for bit, tests/test_configured.py): mu 0.7 > tan 30 holds the
    # block to a creep, mu 0.1 lets it slide, nothing sinks into the plane
    free, pen_f = _ramp_block_slide(0.0)
    stick, pen_s = _ramp_block_slide(0.7)
    slide, pen_l = _ramp_block_slide(0.1)
    assert free < -0.12
    assert abs(stick) < 0.15 * abs(free)
    assert 0.35 * abs(free) < abs(slide) < 0.7 * abs(free)
    assert min(pen_f, pen_s, pen_l) > -0.002


def test_configured_split_children_claim_their_cells():
    # heavy isolated surface particles split; with split_claim two parents
    # never put children in one cell, so no two particles coincide
    p = workloads.lattice((4, 4, 4), 0.0101, (0.3, 0.3, 0.3), 0.0, 1)
    desc = workloads.box_drop(n_side=2, substeps=4, iters=3, adaptive=1, upsample_per=0, skip=True)
    desc.update(particles=p, n_particles=p.shape[0], boundary=np.zeros((0, 3), np.float32), n_boundary=0,
                gravity=(0.0, 0.0, 0.0))
    desc["masses"] = np.full(p.shape[0], 4.0, np.float32)
    workloads.configure(desc["params"], 0.5, 0.4, [])
    desc["params"].mass_ledger = 1
    o = orc.OracleSystem(desc, fp64=False)
    o.step(1)
    x = o.read(abi.FIELD_POS)
    n = x.shape[0]
    assert n > p.shape[0], "the heavy particles must split"
    d = np.linalg.norm(x[:, None, :] - x[None, :, :], axis=-1) + np.eye(n)
    assert d.min() > 0.0, "two particles coincide"
    o.close()
