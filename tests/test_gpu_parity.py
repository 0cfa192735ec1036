"""CUDA path vs the CPU oracle, through the C ABI (needs a GPU).

Bit-exact always: cell keys, stable sort order, cell start tables, contact
and constraint counts, particle counts, merge/split bookkeeping.
Positions and velocities: bit-exact with math_mode = 1 (transcendentals
evaluated in double and rounded once, as the oracle does).  With
math_mode = 0 (CUDA's cbrtf/expf/norm3df/rsqrtf/acosf, the functions the
reference calls) within max(1e-5 r, 4 ulp of the coordinate), max abs.
"""
import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import abi, workloads
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

R = workloads.REF_RADIUS
TOL = 1e-5 * R


def _pair(desc, fp64=False, mode=1):
    desc["params"].math_mode = mode
    s = gg.GranularSystem(**workloads.system_kwargs(desc), masses=desc.get("masses"), device=0)
    o = orc.OracleSystem(desc, fp64=fp64)
    return s, o


# ------------------------------------------------------------------ grid

@pytest.mark.parametrize("n,seed", [(0, 0), (1, 1), (37, 2), (5000, 3), (200_000, 4)])
def test_grid_bit_exact_random(n, seed):
    rng = np.random.default_rng(seed)
    cs = (25, 19, 31)
    L = 0.0404
    pos = rng.uniform(-0.1, 1.4, (n, 3)).astype(np.float32)
    if n > 10:
        pos[: n // 10] = pos[0]               # many duplicates (same key)
        pos[3] = (np.nan, 0.5, 0.5)           # NaN -> cell 0 (cvt.rzi semantics)
        pos[4] = (L * 3, L * 7, L * 11)       # exactly on cell corners
        pos[5] = (-1e-9, 0.2, 0.2)            # just below zero -> out of grid
        pos[6] = (1e30, 0.1, 0.1)             # saturating conversion
    g = gg.Grid(max(n, 1), cs, L)
    k, sk, pm, cst = g.build(pos)
    ok, osk, opm, ocs = orc.grid_build(pos, cs, L)
    assert np.array_equal(k, ok)
    assert np.array_equal(sk, osk)
    assert np.array_equal(pm, opm)
    assert np.array_equal(cst, ocs)
    g.close()


def test_grid_bit_exact_large_sorted_input():
    # nearly sorted input, the common case after the first step
    rng = np.random.default_rng(7)
    cs = (248, 124, 124)
    L = np.float32(0.00808)
    pos = rng.uniform(0, 1, (1_000_000, 3)).astype(np.float32) * np.array([2, 1, 1], np.float32)
    ok, osk, opm, ocs = orc.grid_build(pos, cs, float(L))
    pos2 = pos[opm] + rng.normal(0, 1e-3, pos.shape).astype(np.float32)
    g = gg.Grid(pos2.shape[0], cs, float(L))
    k, sk, pm, cst = g.build(pos2)
    ok, osk, opm, ocs = orc.grid_build(pos2, cs, float(L))
    assert np.array_equal(sk, osk) and np.array_equal(pm, opm) and np.array_equal(cst, ocs)
    g.close()


# ------------------------------------------------------------------ substeps

def _compare(s, o, step, check_contacts=True, exact=True):
    assert s.size() == o.size(), f"step {step}: particle count {s.size()} vs {o.size()}"
    assert np.array_equal(s.read(gg.FIELD_CELL_KEY), o.read(abi.FIELD_CELL_KEY)), f"step {step}: keys"
    assert np.array_equal(s.read(gg.FIELD_CELL_START), o.read(abi.FIELD_CELL_START)), f"step {step}: cell_start"
    if check_contacts:
        cg, co = s.read(gg.FIELD_CONTACTS), o.read(abi.FIELD_CONTACTS)
        ng, no = s.read(gg.FIELD_NUM_CONSTRAINTS), o.read(abi.FIELD_NUM_CONSTRAINTS)
        assert np.array_equal(cg, co), f"step {step}: contacts differ at {np.nonzero(cg != co)[0][:10]}"
        assert np.array_equal(ng, no), f"step {step}: constraint counts differ"
    pg, po = s.read(gg.FIELD_POS), o.read(abi.FIELD_POS)
    vg, vo = s.read(gg.FIELD_VEL), o.read(abi.FIELD_VEL)
    if exact:
        bad = np.nonzero((pg != po).any(1))[0]
        assert bad.size == 0, f"step {step}: positions differ at {bad[:10]}: {pg[bad[:3]]} vs {po[bad[:3]]}"
        assert np.array_equal(vg, vo), f"step {step}: velocities differ"
        return 0.0, 0.0
    tol = np.maximum(TOL, 4 * np.spacing(np.abs(po).astype(np.float32)))
    err = (np.abs(pg - po) / tol).max() if len(pg) else 0.0
    assert err <= 1.0, f"step {step}: max |dx| / tol = {err:.3g}"
    dt = 1.0 / 240.0
    verr = np.abs(vg - vo).max() if len(vg) else 0.0
    assert verr <= (tol.max() * 2) / dt, f"step {step}: max |dv| = {verr:.3g}"
    return err, verr


def test_box_drop_substeps_match_oracle():
    desc = workloads.box_drop(n_side=12, substeps=4, iters=3)
    s, o = _pair(desc)
    _compare(s, o, 0)
    for k in range(1, 25):
        s.step(1)
        o.step(1)
        _compare(s, o, k)
    assert s.read(gg.FIELD_CONTACTS).sum() > 0, "the test scene must produce contacts"


def _edge_scene(name):
    d = workloads.box_drop(n_side=6, substeps=4, iters=3, adaptive=1, upsample_per=4)
    if name == "no_particles":
        d.update(particles=np.zeros((0, 3), np.float32), n_particles=0, upsampled=None, n_upsampled=0)
    elif name == "one_particle":
        p = np.array([[0.5, 0.3, 0.5]], np.float32)
        d.update(particles=p, n_particles=1, upsampled=np.repeat(p, 4, 0) + np.float32(0.001), n_upsampled=4)
    elif name == "all_out_of_grid":
        # the block starts below the grid (y < 0): every key is the
        # out-of-grid sentinel, nothing meets a wall or a partner
        p = d["particles"].copy()
        p[:, 1] -= 1.0
        d.update(particles=p, upsampled=None, n_upsampled=0)
    elif name == "no_walls":
        d.update(boundary=np.zeros((0, 3), np.float32), n_boundary=0)
    elif name == "ragged_cells":
        # a few particles far apart, one dense clump and one on the grid's
        # upper corner: cells of 0, 1 and many particles side by side
        rng = np.random.default_rng(5)
        clump = (np.float32(0.5) + rng.uniform(-0.012, 0.012, (40, 3))).astype(np.float32)
        lone = np.array([[0.1, 0.9, 0.1], [0.9, 0.5, 0.9], [0.999, 0.999, 0.999]], np.float32)
        p = np.concatenate([clump, lone])
        d.update(particles=p, n_particles=p.shape[0],
                 upsampled=np.repeat(p, 4, 0) + np.float32(0.002), n_upsampled=4 * p.shape[0])
    return d


@pytest.mark.parametrize("name", ["no_particles", "one_particle", "all_out_of_grid", "no_walls", "ragged_cells"])
def test_edge_scenes_match_oracle(name):
    # empty and ragged inputs through the whole substep (grid, sweeps,
    # upsampling, merge/split), bit-exact against the oracle
    s, o = _pair(_edge_scene(name))
    _compare(s, o, 0)
    for k in range(1, 7):
        s.step(1)
        o.step(1)
        _compare(s, o, k)
        assert s.upsampled_size() == o.size(abi.SET_UPSAMPLED)
        if s.upsampled_size():
            assert np.array_equal(s.read(gg.FIELD_POS, gg.SET_UPSAMPLED), o.read(abi.FIELD_POS, abi.SET_UPSAMPLED))


@pytest.mark.parametrize("variant,lists", [(0, True), (0, False), (1, True)])
def test_sweep_variants_bit_exact(variant, lists):
    # the sweep kernels (kernels_sweep.cu): contact lists (default), the
    # 27-cell listed scan without lists (nlist_skin = 0), and the pruned
    # one-thread-per-particle scan (gg_tuning.sweep_variant = 1)
    desc = workloads.box_drop(n_side=16, substeps=4, iters=5, adaptive=1, upsample_per=2)
    if not lists:
        desc["params"].nlist_skin = 0.0
    s, o = _pair(desc)
    s.set_tuning(sweep_variant=variant)
    assert s.tuning()["sweep_variant"] == variant
    for k in range(1, 8):
        s.step(1)
        o.step(1)
        _compare(s, o, k)


@pytest.mark.parametrize("skin", [0.4 * R, 1e-4 * R, 3.0 * R])
def test_listed_sweep_bit_exact(skin):
    # contact lists reused across sweeps; the tiny skin forces rebuilds and
    # the large one overflows the lists (full scans)
    desc = workloads.box_drop(n_side=16, substeps=4, iters=5, adaptive=1, upsample_per=2)
    desc["params"].nlist_skin = skin
    s, o = _pair(desc)
    sweeps = desc["params"].stab_iters + desc["params"].iters
    built = 0
    scanned = 0
    for k in range(1, 10):
        n = s.size()
        s.profile_begin()
        s.step(1)
        built += s.profile_end()["_nlist_rebuilds"]
        scanned += n * sweeps
        o.step(1)
        _compare(s, o, k)
    if skin < R:
        # every sweep scans with the tiny skin; the usual one keeps lists
        assert (built == scanned) if skin < 1e-3 * R else (built < scanned / 2)


def test_sweep_column_scene_bit_exact():
    # the benchmark scene's geometry (walls, 2x1x1 box, r = 0.002) at a size
    # the oracle finishes quickly
    desc = workloads.column_collapse(counts=(24, 40, 32), upsample_per=2)
    desc["params"].nlist_skin = 0.4 * 0.002
    s, o = _pair(desc)
    for k in range(1, 5):
        s.step(1)
        o.step(1)
        _compare(s, o, k)


def test_box_drop_cuda_math_within_ulps():
    # CUDA's own transcendentals (the reference's): one substep from an
    # identical input state lands within max(1e-5 r, 4 ulp) of the oracle
    desc = workloads.box_drop(n_side=12, substeps=4, iters=3)
    s, o = _pair(desc, mode=0)
    for k in range(1, 8):
        o.write(abi.FIELD_POS, s.read(gg.FIELD_POS))
        o.write(abi.FIELD_VEL, s.read(gg.FIELD_VEL))
        s.step(1)
        o.step(1)
        _compare(s, o, k, exact=False)


def test_reference_iteration_counts_and_upsampling():
    desc = workloads.box_drop(n_side=9, substeps=4, iters=5, upsample_per=6)
    s, o = _pair(desc)
    for k in range(12):
        s.step(1)
        o.step(1)
        _compare(s, o, k)
        ug, uo = s.read(gg.FIELD_POS, gg.SET_UPSAMPLED), o.read(abi.FIELD_POS, abi.SET_UPSAMPLED)
        assert np.array_equal(ug, uo)
        vg, vo = s.read(gg.FIELD_VEL, gg.SET_UPSAMPLED), o.read(abi.FIELD_VEL, abi.SET_UPSAMPLED)
        assert np.array_equal(vg, vo)


@pytest.mark.parametrize("ledger,mixed", [(0, False), (1, False), (0, True), (1, True)])
def test_adaptive_merge_split_match_oracle(ledger, mixed):
    # mixed: masses drawn from 1, 1.5, 2 and 3, so that the merge density
    # (an average mass) and the merge velocity depend on which neighbours
    # are summed, and heavy surface particles split
    desc = workloads.box_drop(n_side=14, substeps=4, iters=5, adaptive=1, upsample_per=2)
    desc["params"].mass_ledger = ledger
    if mixed:
        rng = np.random.default_rng(9)
        desc["masses"] = rng.choice(np.array([1.0, 1.0, 1.5, 2.0, 3.0], np.float32), desc["n_particles"])
    s, o = _pair(desc)
    for k in range(1, 56):
        s.step(1)
        o.step(1)
        _compare(s, o, k)
        for f in (gg.FIELD_REMOVE, gg.FIELD_MERGE_COUNT, gg.FIELD_SURFACE, gg.FIELD_ADAPTIVE_LAST_STEP,
                  gg.FIELD_MERGE, gg.FIELD_MERGE_VELOCITY):
            a, b = s.read(f), o.read(f)
            assert np.array_equal(a, b), f"step {k}: field {f} differs"
        assert np.array_equal(s.read(gg.FIELD_MASS), o.read(abi.FIELD_MASS)), f"step {k}: masses"
        if ledger:
            assert np.array_equal(s.read(gg.FIELD_MASS_UNITS), o.read(abi.FIELD_MASS_UNITS))
    st = s.stats()
    assert st["merged_total"] > 0, "scene must merge within 55 steps (first merge completes at step 40)"
    if ledger:
        m0 = desc.get("masses")
        total = desc["n_particles"] if m0 is None else float(np.sum(m0, dtype=np.float64))
        assert st["total_mass_units"] == round(total * abi.UNITS_PER_MASS)


def test_ledger_conserves_mass_exactly_through_merge_and_split():
    desc = workloads.box_drop(n_side=16, substeps=4, iters=5, adaptive=1)
    desc["params"].mass_ledger = 1
    desc["params"].max_mass = 8.0
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    total = desc["n_particles"] * abi.UNITS_PER_MASS
    merged = 0
    for _ in range(90):
        s.step(1)
        u = s.read(gg.FIELD_MASS_UNITS)
        assert int(u.astype(np.int64).sum()) == total
        merged += s.stats()["merged_last"]
    assert merged > 0


def test_scene_json_path_matches_oracle(tmp_path):
    scene = tmp_path / "box_small.json"
    scene.write_text("""{
      "space_size": {"x": 1.0, "y": 1.0, "z": 1.0}, "dt": 0.002,
      "gravity": {"x": 0.0, "y": -9.8, "z": 0.0}, "sph_spacing": 0.02, "init_spacing": 0.021,
      "smoothing_radius": 0.04, "cell_length": 0.0404, "density": 238732.4146,
      "box_size": {"x": 9, "y": 8, "z": 7}, "scene": 1,
      "boundary_translation": {"x": 0.0, "y": 0.0, "z": 0.0},
      "particle_translation": {"x": 0.05, "y": 0.0, "z": 0.1},
      "obj_file": "", "is_adaptive": 1, "save_file": "unused"}""")
    sc = gg.scene_build(str(scene))
    prm = abi.default_params()
    prm.math_mode = 1
    sc["params"] = prm
    s = gg.GranularSystem.from_scene(str(scene), params=prm)
    desc = dict(particles=sc["particles"], n_particles=len(sc["particles"]), boundary=sc["boundary"],
                n_boundary=len(sc["boundary"]), boundary_animated=sc["boundary_animated"],
                upsampled=sc["upsampled"], n_upsampled=len(sc["upsampled"]), space_size=sc["space_size"],
                cell_length=sc["cell_length"], dt=sc["dt"], gravity=sc["gravity"], cell_size=sc["cell_size"],
                density=sc["density"], upsampled_radius=sc["upsampled_radius"],
                is_move_boundary=sc["is_move_boundary"], is_adaptive=sc["is_adaptive"], skip_initial_step=0,
                device=0, max_particles=0, params=sc["params"])
    o = orc.OracleSystem(desc)
    assert s.size() == 9 * 8 * 7 and s.upsampled_size() == 25 * 9 * 8 * 7
    for k in range(6):
        _compare(s, o, k)
        s.step(1)
        o.step(1)


def test_snapshot_round_trip(tmp_path):
    desc = workloads.box_drop(n_side=8, substeps=4, iters=3, adaptive=1, upsample_per=2)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    s.step(3)
    path = str(tmp_path / "snap.bin")
    s.save(path)
    s.step(4)
    a = s.read(gg.FIELD_POS)
    s.load(path)
    s.step(4)
    b = s.read(gg.FIELD_POS)
    assert np.array_equal(a, b)


def test_stats_and_explosion():
    desc = workloads.box_drop(n_side=8, substeps=4, iters=3)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    st = s.stats()
    m = s.read(gg.FIELD_MASS).astype(np.float64)
    p = s.read(gg.FIELD_POS).astype(np.float64)
    assert st["total_mass"] == pytest.approx(m.sum(), rel=1e-12)
    com = (m[:, None] * p).sum(0) / m.sum()
    assert np.allclose(st["center_of_mass"], com, rtol=1e-9, atol=1e-12)
    assert st["nonfinite"] == 0
    v0 = s.read(gg.FIELD_VEL).astype(np.float64)
    s.get_solver().trigger_explosion(1.0)
    v1 = s.read(gg.FIELD_VEL).astype(np.float64)
    d = p - com
    dist = np.linalg.norm(d, axis=1)
    expect = v0 + d / dist[:, None] * (1.0 / (1.0 + dist ** 2))[:, None] / m[:, None]
    assert np.abs(v1 - expect).max() < 1e-4


def test_frame_times_and_profile():
    desc = workloads.box_drop(n_side=8, substeps=4, iters=3)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    s.set_frame_timing(True)
    s.profile_begin()
    s.step(3)
    prof = s.profile_end()
    ft = s.get_frame_times()
    assert len(ft) == 3 and (ft > 0).all()
    assert prof["sweep"]["launches"] == 3 * 6 and prof["sweep"]["ms"] > 0


def _split_scene(n_side=5, mass=4.0, max_particles=0):
    # sparse heavy particles: every one is a surface particle with empty
    # neighbour cells, so each splits at its first adaptive step
    base = workloads.box_drop(n_side=2, substeps=4, iters=3, adaptive=1)
    p = workloads.lattice((n_side,) * 3, 0.13, (0.2, 0.35, 0.2), 0.002, 5)
    base.update(particles=p, n_particles=p.shape[0], masses=np.full(p.shape[0], mass, np.float32),
                max_particles=max_particles)
    return base


@pytest.mark.parametrize("ledger", [0, 1])
def test_split_children_match_oracle(ledger):
    desc = _split_scene()
    desc["params"].mass_ledger = ledger
    desc["params"].math_mode = 1
    s = gg.GranularSystem(**workloads.system_kwargs(desc), masses=desc["masses"], device=0)
    o = orc.OracleSystem(desc)
    n0 = desc["n_particles"]
    assert s.size() > n0, "every heavy surface particle splits in the constructor's step"
    for k in range(8):
        _compare(s, o, k)
        assert np.array_equal(s.read(gg.FIELD_MASS), o.read(abi.FIELD_MASS))
        s.step(1)
        o.step(1)
    if ledger:
        assert int(s.read(gg.FIELD_MASS_UNITS).astype(np.int64).sum()) == n0 * 4 * abi.UNITS_PER_MASS


def test_capacity_overflow_is_reported_and_drops_children():
    desc = _split_scene(n_side=4, max_particles=64 + 5)
    desc["skip_initial_step"] = 1
    s = gg.GranularSystem(**workloads.system_kwargs(desc), masses=desc["masses"], device=0)
    with pytest.raises(gg.GranularError) as ei:
        s.step(1)
    assert ei.value.status == abi.GG_ERR_CAPACITY


def test_capacity_overflow_matches_oracle_survivors():
    desc = _split_scene(n_side=4, max_particles=64 + 5)
    desc["skip_initial_step"] = 1
    desc["params"].math_mode = 1
    s = gg.GranularSystem(**workloads.system_kwargs(desc), masses=desc["masses"], device=0)
    o = orc.OracleSystem(desc)
    with pytest.raises(gg.GranularError):
        s.step(1)
    o.step(1)
    assert s.size() == o.size() == 69
    assert np.array_equal(s.read(gg.FIELD_POS), o.read(abi.FIELD_POS))
    assert np.array_equal(s.read(gg.FIELD_MASS), o.read(abi.FIELD_MASS))


def test_vtk_writer(tmp_path):
    desc = workloads.box_drop(n_side=5, substeps=4, iters=3, upsample_per=2)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    path = tmp_path / "frame.vtk"
    s.write_vtk(str(path))
    lines = path.read_text().splitlines()
    n = s.upsampled_size()
    assert lines[0] == "# vtk DataFile Version 3.0" and lines[4] == f"POINTS {n} float"
    x = s.read(gg.FIELD_POS, gg.SET_UPSAMPLED)
    first = [float(v) for v in lines[5].split()]
    assert np.allclose(first, [x[0, 0], x[0, 2], x[0, 1]], rtol=1e-5)
    assert lines[5 + n] == f"CELLS {n} {2 * n}" and lines[6 + 2 * n] == f"CELL_TYPES {n}"


def test_host_copies_pinned_misaligned_and_pageable_agree():
    # pinned buffers are packed by the copy kernel itself, pageable ones go
    # through the device staging buffer: every path returns and accepts the
    # same bits, aligned or not, including a partial last block
    torch = pytest.importorskip("torch")
    desc = workloads.box_drop(n_side=11, upsample_per=2)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    s.step(2)
    n = s.size()
    assert n % 256 != 0 and n > 256
    ref = s.read(gg.FIELD_POS).copy()
    refu = s.read(gg.FIELD_VEL, gg.SET_UPSAMPLED).copy()
    pin = torch.empty(3 * n + 1, dtype=torch.float32, pin_memory=True).numpy()
    aligned, shifted = pin[: 3 * n].reshape(n, 3), pin[1: 3 * n + 1].reshape(n, 3)
    for buf in (aligned, shifted):
        buf[:] = 0
        s.read(gg.FIELD_POS, out=buf)
        assert np.array_equal(buf, ref)
    nu = refu.shape[0]
    upin = torch.empty((nu, 3), dtype=torch.float32, pin_memory=True).numpy()
    s.read(gg.FIELD_VEL, gg.SET_UPSAMPLED, out=upin)
    assert np.array_equal(upin, refu)
    moved = ref + np.float32(1e-3)
    for buf in (np.array(ref), aligned, shifted):
        buf[:] = moved
        s.write(gg.FIELD_POS, buf)
        assert np.array_equal(s.read(gg.FIELD_POS), moved)
    s.close()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_color_buffer_matches_oracle(mode):
    desc = workloads.box_drop(n_side=12, substeps=4, iters=5, adaptive=1, upsample_per=2)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    s.step(45)
    for which in (gg.SET_GRANULAR, gg.SET_UPSAMPLED):
        dots, cols = s.color_buffer(mode, which, 1.0, 4.0)
        if which == gg.SET_GRANULAR:
            od, oc = orc.color_dots(s.read(gg.FIELD_POS), s.read(gg.FIELD_MASS), s.read(gg.FIELD_SURFACE),
                                    s.read(gg.FIELD_SURFACE_DISTANCE), mode, 1.0, 4.0)
        else:
            od, oc = orc.color_dots(s.read(gg.FIELD_POS, gg.SET_UPSAMPLED), mode=mode)
        assert np.array_equal(dots, od) and np.array_equal(cols, oc), which
    with pytest.raises(gg.GranularError):
        s.color_buffer(3)
    s.close()


@pytest.mark.parametrize("law", ["cap", "coulomb"])
def test_residual_mode_lists_match_the_stencil_scan(law):
    # residual mode: every Jacobi sweep writes the counts, and each sweep's
    # per-cell increments still bound the next sweep's contact lists; the
    # listed sweeps equal the 27-cell scan without lists bit for bit
    from granular_gpu_gb300 import learn as L
    out = []
    for skin in (-1.0, 0.0):
        desc = L.pile_scene(6, dims=(0.2, 0.15, 0.2), drop=0.01, target_residual=1e-3 * L.R, max_sweeps=120,
                            law=law)
        desc["params"].nlist_skin = skin
        s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
        sweeps = 0
        for _ in range(12):
            s.step(1)
            sweeps += s.stats()["last_sweeps"]
        out.append((s.read(gg.FIELD_POS), s.read(gg.FIELD_VEL), s.read(gg.FIELD_NUM_CONSTRAINTS), sweeps))
        s.close()
    assert out[0][3] == out[1][3] and out[0][3] > 12
    for a, b in zip(out[0][:3], out[1][:3]):
        assert np.array_equal(a, b)
