"""The CUDA path against the reference's own CUDA kernels (needs a GPU).

`oracle/ref_cuda_build.py` compiles the reference's `src/Solver.cu` and
`src/GranularSystem.cu` into cubins; `oracle/ref_cuda.py` runs their
`__global__` kernels through the CUDA driver API and restates the host code
around them.  From one state read out of this library, both run and are
compared.  "nofma" is the reference built with -fmad=false (every operation
rounds as written, as in this library's build); "own flags" is the
reference's own build, which contracts multiply-adds.

Deterministic reference kernels, bit-exact against nofma and within
1e-5 r against the own-flags build:
* grid keys, stable order and cell start tables;
* a substep of a scene whose contacts are all with the walls, and of a
  scene of isolated particle pairs (no contact races);
* the upsampling kernel and the surface / distance kernels, fed the same
  granular state.

The reference's contact kernel (`compute_delta_pos`, `src/Solver.cu:361-401`)
races: corrections and constraint counts are scattered to neighbours with
plain read-modify-writes, and each thread's final `delta_pos[i] = dp`
overwrites scatters that landed earlier.  Its output changes from run to run.
This library implements one legal schedule of that kernel (every neighbour
loop runs before any final store, no increment is lost).  For dense scenes
the tests therefore check what holds under every schedule:
* in one sweep the reference's count n_i never exceeds this library's
  (contacts i finds + particles that find i, i.e. no increment lost), and
  rarely falls below the contacts i finds itself;
* after a substep this library is as close to the reference as two runs of
  the reference are to each other (within a small factor);
* over a long run, centre of mass and kinetic energy follow the reference's.
"""
import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import workloads

pytestmark = pytest.mark.gpu

ref_cuda = pytest.importorskip("oracle.ref_cuda")
if not ref_cuda.available():
    pytest.skip("the reference's kernels were not built (no reference checkout where they were compiled)",
                allow_module_level=True)

R = workloads.REF_RADIUS
TOL = 1e-5 * R


@pytest.fixture(scope="module")
def kernels():
    k = {False: ref_cuda.RefKernels(fma=False), True: ref_cuda.RefKernels(fma=True)}
    yield k
    for v in k.values():
        v.close()


def _t(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), device="cuda").contiguous()


@pytest.mark.parametrize("n,seed", [(1, 1), (37, 2), (5000, 3), (200_000, 4)])
def test_grid_matches_reference_kernels(kernels, n, seed):
    import torch
    rng = np.random.default_rng(seed)
    cs = (25, 19, 31)
    L = np.float32(0.0404)
    pos = rng.uniform(-0.1, 1.4, (n, 3)).astype(np.float32)
    if n > 10:
        pos[: n // 10] = pos[0]
        pos[3] = (np.nan, 0.5, 0.5)
        pos[4] = (L * 3, L * 7, L * 11)
        pos[5] = (-1e-9, 0.2, 0.2)
        pos[6] = (1e30, 0.1, 0.1)
    k = kernels[True]
    sysr = ref_cuda.RefSystem(k, pos[:1], np.zeros((1, 3)), np.ones(1), pos[:1], cell_size=cs,
                              cell_length=L, dt=0.01, gravity=(0, -9.81, 0), density=1.0)
    rkeys = sysr.keys(_t(pos))
    rsk, rperm = torch.sort(rkeys, stable=True)
    rcs = sysr.cell_start(rsk)
    k.synchronize()
    g = gg.Grid(max(n, 1), cs, float(L))
    keys, sk, perm, cst = g.build(pos)
    g.close()
    assert np.array_equal(keys, rkeys.cpu().numpy())
    assert np.array_equal(sk, rsk.cpu().numpy())
    assert np.array_equal(perm, rperm.cpu().numpy().astype(np.int32))
    assert np.array_equal(cst, rcs.cpu().numpy())
    # the CPU oracle's grid build against the same reference kernels
    from oracle import oracle as orc
    ok, osk, opm, ocs = orc.grid_build(pos, cs, float(L))
    assert np.array_equal(ok, rkeys.cpu().numpy()) and np.array_equal(ocs, rcs.cpu().numpy())
    assert np.array_equal(opm, rperm.cpu().numpy().astype(np.int32))


def _ref_from(k, s, desc, adaptive=False):
    up = s.upsampled_size() > 0
    r = ref_cuda.RefSystem(
        k, s.read(gg.FIELD_POS), s.read(gg.FIELD_VEL), s.read(gg.FIELD_MASS), s.read(gg.FIELD_POS, gg.SET_BOUNDARY),
        s.read(gg.FIELD_POS, gg.SET_UPSAMPLED) if up else None, s.read(gg.FIELD_VEL, gg.SET_UPSAMPLED) if up else None,
        cell_size=desc["cell_size"], cell_length=desc["cell_length"], dt=desc["dt"], gravity=desc["gravity"],
        density=desc["density"], max_iter=desc["params"].iters, stab_iters=desc["params"].stab_iters,
        adaptive=adaptive)
    # adaptive_last_step stays with its slot through the sort, as in the reference
    r.set_adaptive_last_step(s.read(gg.FIELD_ADAPTIVE_LAST_STEP))
    return r


def _ndiff(a, b):
    a, b = np.asarray(a), np.asarray(b)
    bad = (a != b).any(1) if a.ndim == 2 else (a != b)
    return int(bad.sum())


def _maxabs(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.abs(a - b).max()) if a.size else 0.0


def _box(n_side=10, upsample_per=0, adaptive=0, stab=3, iters=5):
    desc = workloads.box_drop(n_side=n_side, substeps=4, iters=iters, adaptive=adaptive,
                              upsample_per=upsample_per)
    desc["params"].stab_iters = stab
    desc["params"].math_mode = 0  # CUDA's own cbrtf/expf/norm3df, the functions the reference calls
    return desc


def _check_step(kernels, desc, fields=("pos", "vel", "last_n")):
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    refs = {fma: _ref_from(kernels[fma], s, desc) for fma in (False, True)}
    s.step(1)
    for r in refs.values():
        r.step()
    ours = {"pos": s.read(gg.FIELD_POS), "vel": s.read(gg.FIELD_VEL),
            "last_n": s.read(gg.FIELD_NUM_CONSTRAINTS)}
    contacts = int(s.read(gg.FIELD_CONTACTS).sum())
    for f in fields:
        nb = _ndiff(ours[f], refs[False].read(f))
        assert nb == 0, f"{f}: {nb} particles differ from the reference (-fmad=false), " \
                        f"max {_maxabs(ours[f], refs[False].read(f)):.3g}"
    e = _maxabs(ours["pos"], refs[True].read("pos"))
    assert e <= TOL, f"positions vs the reference's own build: max |dx| {e:.3g}"
    s.close()
    return contacts


@pytest.mark.parametrize("stab,iters", [(1, 0), (3, 5)])
def test_wall_contacts_match_reference_build(kernels, stab, iters):
    # lattice at spacing 3r (no particle pairs touch), bottom layer 0.018
    # above the floor walls (wall contact distance 0.02)
    desc = _box(n_side=8, stab=stab, iters=iters)
    p = desc["particles"]
    c = p.mean(0)
    p = (p - c) * 1.5 + c
    p[:, 1] += 0.023 - p[:, 1].min()
    desc["particles"] = p.astype(np.float32)
    assert _check_step(kernels, desc) > 0


@pytest.mark.parametrize("stab,iters", [(1, 0), (3, 5)])
def test_isolated_pairs_match_reference_build(kernels, stab, iters):
    # 512 pairs at distance 0.95 (r_i + r_j), pair centres 3 cells apart
    rng = np.random.default_rng(5)
    centres = workloads.lattice((8, 8, 8), 0.06, (0.3, 0.3, 0.3), 0.0, 0)
    d = rng.normal(size=(centres.shape[0], 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    desc = _box(n_side=8, stab=stab, iters=iters)
    desc["particles"] = np.concatenate([centres + 0.0095 * d, centres - 0.0095 * d]).astype(np.float32)
    desc["n_particles"] = desc["particles"].shape[0]
    desc["skip_initial_step"] = 1
    _check_step(kernels, desc)


@pytest.mark.parametrize("scene", ["box", "column"])
def test_upsampling_kernel_matches_reference(kernels, scene):
    # box: r = 0.01, the support 0.045 reaches part of the stencil (masked
    # scan); column: r = 0.002 with the reference's constants, the support
    # covers the whole stencil (two points per thread, packed arithmetic)
    if scene == "box":
        desc = _box(n_side=10, upsample_per=4)
        pre = 70  # landed and piling
    else:
        # no merge/split: the velocities and positions read after the step are
        # the ones the upsampling saw
        desc = workloads.column_collapse(counts=(16, 32, 32), constants="reference", upsample_per=5, adaptive=0)
        desc["params"].math_mode = 0
        pre = 30  # collapsing
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    s.step(pre)
    refs = {fma: _ref_from(kernels[fma], s, desc) for fma in (False, True)}
    for r in refs.values():
        r.neighbor_search()  # the step-start grids the kernel reads
    s.step(1)
    for r in refs.values():
        r.pos, r.vel = _t(s.read(gg.FIELD_POS)), _t(s.read(gg.FIELD_VEL))
        r.upsampled_update()
        r.k.synchronize()
    ug, uvg = s.read(gg.FIELD_POS, gg.SET_UPSAMPLED), s.read(gg.FIELD_VEL, gg.SET_UPSAMPLED)
    assert _ndiff(ug, refs[False].read("upos")) == 0
    assert _ndiff(uvg, refs[False].read("uvel")) == 0
    assert _maxabs(ug, refs[True].read("upos")) <= TOL
    s.close()


def test_surface_kernels_match_reference(kernels):
    desc = _box(n_side=12, adaptive=1)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    checked = blended = 0
    for step in range(1, 92):
        compare = step in (3, 10, 20, 30, 40, 45, 60, 75, 90)
        if compare:
            ref = _ref_from(kernels[False], s, desc, adaptive=True)
            ref.neighbor_search()
            m0 = ref.mass.clone()
        n0 = s.size()
        s.step(1)
        if not compare or s.size() != n0:
            continue  # compare only steps that neither remove nor append particles
        ref.pos, ref.mass = _t(s.read(gg.FIELD_POS)), m0
        ref.surface_pass()
        ref.k.synchronize()
        sg, sr = s.read(gg.FIELD_SURFACE), ref.read("surface")
        dg, dr = s.read(gg.FIELD_SURFACE_DISTANCE), ref.read("surface_distance")
        assert _ndiff(sg, sr) == 0, f"step {step}: {_ndiff(sg, sr)} of {len(sg)} surface flags differ"
        assert _ndiff(dg, dr) == 0, f"step {step}: {_ndiff(dg, dr)} distances differ"
        assert 0 < sg.sum() < len(sg)
        checked += 1
        blended += int((ref.read("mass") != 1.0).sum())
    assert checked >= 3 and blended > 0, (checked, blended)
    s.close()


def test_racy_sweep_counts_within_every_schedule(kernels):
    # one sweep of a jittered lattice: dense contacts, racy scatters
    desc = _box(n_side=10, stab=1, iters=0)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    refs = [_ref_from(kernels[False], s, desc) for _ in range(3)]
    s.step(1)
    for r in refs:
        r.step()
    ours, own = s.read(gg.FIELD_NUM_CONSTRAINTS), s.read(gg.FIELD_CONTACTS)
    assert own.sum() > 500
    for r in refs:
        rn = r.read("last_n")
        assert (rn <= ours).all(), f"reference count above the no-lost-update count at {np.nonzero(rn > ours)[0][:8]}"
        assert (rn >= own).mean() >= 0.99
    s.close()


@pytest.mark.parametrize("pre_steps", [0, 80])
def test_substep_within_reference_self_spread(kernels, pre_steps):
    desc = _box(n_side=10)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    if pre_steps:
        s.step(pre_steps)
    refs = [_ref_from(kernels[False], s, desc) for _ in range(4)]
    s.step(1)
    for r in refs:
        r.step()
    pg = s.read(gg.FIELD_POS)
    P = [r.read("pos") for r in refs]
    self_spread = max(_maxabs(P[a], P[b]) for a in range(4) for b in range(a + 1, 4))
    ours = max(_maxabs(pg, p) for p in P)
    print(f"pre_steps {pre_steps}: reference self-spread {self_spread / R:.3g} r, ours vs reference {ours / R:.3g} r")
    assert self_spread > 0, "the reference's contact kernel is expected to race on a dense scene"
    assert ours <= 4.0 * self_spread
    s.close()


def _low_box(stab=3, iters=5):
    # the box-drop block with its bottom layer 0.03 above the floor: it
    # lands slowly enough that no particle passes through the walls
    desc = _box(n_side=10, stab=stab, iters=iters)
    p = desc["particles"]
    p[:, 1] += np.float32(0.03) - p[:, 1].min()
    desc["particles"] = p
    return desc


@pytest.mark.parametrize("pre_steps", [0, 40])
def test_sweep_correction_magnitude_vs_reference(kernels, pre_steps):
    # The reference loses some of the racy count increments, so its
    # divisor n_i is smaller than this library's and its mean correction per
    # sweep larger: by 14-18 % on these scenes.  The bound pins that gap.
    desc = _low_box(stab=1, iters=0)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    if pre_steps:
        s.step(pre_steps)
    x0, v0 = s.read(gg.FIELD_POS), s.read(gg.FIELD_VEL)
    refs = [_ref_from(kernels[False], s, desc) for _ in range(3)]
    s.step(1)
    for r in refs:
        r.step()
    dt = np.float32(desc["dt"])
    xs = x0 + dt * (v0 + dt * np.array(desc["gravity"], np.float32))  # x* of the predict
    ours = np.linalg.norm(s.read(gg.FIELD_POS) - xs, axis=1).mean()
    for r in refs:
        ratio = np.linalg.norm(r.read("pos") - xs, axis=1).mean() / ours
        print(f"pre_steps {pre_steps}: mean correction, reference / this library = {ratio:.3f}")
        assert 1.0 <= ratio <= 1.35
    s.close()


def test_long_run_statistics_follow_reference(kernels):
    # 300 substeps (1.25 s) of a low drop that settles into a pile: centre of
    # mass, pile height and resting kinetic energy of this library against
    # the reference run from the same initial state, next to the spread of
    # two reference runs
    desc = _low_box()
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    refs = [_ref_from(kernels[False], s, desc) for _ in range(2)]
    com = {k: [] for k in ("ours", 0, 1)}
    ke = {k: [] for k in ("ours", 0, 1)}
    for _ in range(300):
        s.step(1)
        for r in refs:
            r.step()
        for key, p, v in (("ours", s.read(gg.FIELD_POS), s.read(gg.FIELD_VEL)),
                          (0, refs[0].read("pos"), refs[0].read("vel")),
                          (1, refs[1].read("pos"), refs[1].read("vel"))):
            com[key].append(p.astype(np.float64).mean(0))
            ke[key].append(0.5 * float((v.astype(np.float64) ** 2).sum()))
    c = {k: np.array(v) for k, v in com.items()}
    e = {k: np.array(v) for k, v in ke.items()}
    d_ours = np.abs(c["ours"] - c[0]).max()
    d_ref = np.abs(c[1] - c[0]).max()
    print(f"centre of mass: ours vs reference {d_ours / R:.3g} r, reference vs reference {d_ref / R:.3g} r")
    assert d_ours <= max(5.0 * d_ref, 1.5 * R)
    h = abs(c["ours"][-1, 1] - c[0][-1, 1])
    print(f"pile centre height: ours vs reference {h / R:.3g} r")
    assert h <= 0.3 * R
    rest = {k: v[-100:].mean() for k, v in e.items()}
    print(f"resting kinetic energy: ours {rest['ours']:.4g}, reference {rest[0]:.4g} and {rest[1]:.4g}")
    # the racy reference's own resting energy varies by a factor of two
    # between runs: compare with the range of both
    assert 0.5 * min(rest[0], rest[1]) <= rest["ours"] <= 2.0 * max(rest[0], rest[1])
    s.close()


def _pile_shape(p):
    # (angle in degrees, median reach, 95th-percentile reach): the cone
    # through the particles' 95th-percentile height above the lowest one and
    # their 95th-percentile horizontal distance from the vertical axis through
    # their centre; the median distance measures the bulk, the 95th
    # percentile the particles splashed across the floor
    p = p.astype(np.float64)
    d = np.hypot(p[:, 0] - p[:, 0].mean(), p[:, 2] - p[:, 2].mean())
    h = p[:, 1] - p[:, 1].min()
    reach = float(np.percentile(d, 95))
    return float(np.degrees(np.arctan2(np.percentile(h, 95), reach))), float(np.median(d)), reach


def test_pile_shape_follows_reference(kernels):
    # a 6 x 30 x 6 column dropped from 0.25 m lands on the floor (500
    # substeps, about 2 s).  In the reference's model a landed stack barely
    # slumps: the mass scaling m exp(-y) makes lower particles heavier and
    # speeds below 0.01 are zeroed every substep, so the column stays steep.
    # Its profile angle and reach against the reference's from the same
    # initial state, next to the spread of two reference runs.
    desc = _box(n_side=10)
    r = workloads.REF_RADIUS
    col = workloads.lattice((6, 30, 6), 2 * r, (0.5 - 5 * r, 0.25, 0.5 - 5 * r), 0.05 * r, 7)
    desc["particles"], desc["n_particles"] = col, col.shape[0]
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    refs = [_ref_from(kernels[False], s, desc) for _ in range(2)]
    for _ in range(500):
        s.step(1)
        for ref in refs:
            ref.step()
    a, med, reach = _pile_shape(s.read(gg.FIELD_POS))
    b = [_pile_shape(ref.read("pos")) for ref in refs]
    print(f"profile angle: ours {a:.2f} deg, reference {b[0][0]:.2f} and {b[1][0]:.2f} deg; "
          f"median reach: ours {med / r:.2f} r, reference {b[0][1] / r:.2f} and {b[1][1] / r:.2f} r; "
          f"95th-percentile reach: ours {reach / r:.2f} r, reference {b[0][2] / r:.2f} and {b[1][2] / r:.2f} r")
    assert abs(a - b[0][0]) <= max(3.0 * abs(b[1][0] - b[0][0]), 1.0), (a, b)
    assert abs(med - b[0][1]) <= max(3.0 * abs(b[1][1] - b[0][1]), 0.15 * b[0][1]), (med, b)
    # the splash reaches further here: this library's sweep corrects about
    # 15 % less than the reference's racy one (it loses no count increments)
    assert 0.7 * b[0][2] <= reach <= 1.4 * b[0][2], (reach, b)
    s.close()


@pytest.mark.parametrize("counts", [(64, 128, 128), (128, 256, 256)])
def test_throughput_against_reference_kernels(kernels, counts):
    """Substep time of this library against the reference's own kernels
    (own flags, driven by the harness's host restatement) on the column
    collapse without merge/split, upsampling on, the reference's constants
    as compiled in: this library must be at least 1.5x as fast."""
    import torch
    desc = workloads.column_collapse(counts=counts, adaptive=0, upsample_per=4)
    p = workloads.scaled_params(workloads.REF_RADIUS, iters=5)
    p.upsample_enabled, p.merge_enabled, p.math_mode = 1, 0, 0
    desc["params"] = p
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    s.step(2)
    ref = _ref_from(kernels[True], s, desc)
    ref.step()
    K = 3
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(K):
        ref.step()
    e1.record()
    e1.synchronize()
    ms_ref = e0.elapsed_time(e1) / K
    st = torch.cuda.ExternalStream(s.stream)
    s.synchronize()
    e0.record(st)
    for _ in range(K):
        s.step(1)
    e1.record(st)
    e1.synchronize()
    ms_ours = e0.elapsed_time(e1) / K
    print(f"{desc['n_particles']} particles, {desc['n_upsampled']} render points: reference kernels "
          f"{ms_ref:.1f} ms per substep, this library {ms_ours:.2f} ms: {ms_ref / ms_ours:.1f}x")
    assert ms_ref / ms_ours >= 1.5
    s.close()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_color_buffer_matches_reference_kernel(kernels, mode):
    # generate_dots_CUDA (VBO.hpp) on the same state: particles after merges
    # have started (blended masses, surface flags and distances), render
    # points with the reference's zero-filled mass, surface and distance
    import torch
    desc = _box(n_side=12, upsample_per=2, adaptive=1)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    s.step(45)
    masses = s.read(gg.FIELD_MASS)
    assert (masses != 1.0).any()
    for which in (gg.SET_GRANULAR, gg.SET_UPSAMPLED):
        dots, cols = s.color_buffer(mode, which, 1.0, 4.0)
        n = dots.shape[0]
        pos = _t(s.read(gg.FIELD_POS, which))
        if which == gg.SET_GRANULAR:
            mass, surf = _t(masses), _t(s.read(gg.FIELD_SURFACE).astype(np.int32))
            sd = _t(s.read(gg.FIELD_SURFACE_DISTANCE))
        else:
            mass, sd = torch.zeros(n, device="cuda"), torch.zeros(n, device="cuda")
            surf = torch.zeros(n, dtype=torch.int32, device="cuda")
        for fma in (False, True):
            rd = torch.empty((n, 3), dtype=torch.float32, device="cuda")
            rc = torch.empty_like(rd)
            kernels[fma].launch("generate_dots_CUDA", n, rd, rc, pos, n, surf, mass, 4.0, 1.0, mode, sd)
            kernels[fma].synchronize()
            assert _ndiff(dots, rd.cpu().numpy()) == 0, (which, fma)
            assert _ndiff(cols, rc.cpu().numpy()) == 0, (which, fma)
        if mode == 2 and which == gg.SET_UPSAMPLED:
            assert np.isinf(cols[:, 0]).all()  # mass 0: the reference's 6.0 / 255 / 0
    s.close()
