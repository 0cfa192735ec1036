"""Merge and split against the reference's own kernels, run on the GB300.

`merge_mark_gpu`, `merge_count_gpu`, `check_neighborhood` / `split_gpu` and
`extract_split_particles_kernel` (src/Solver.cu:526-843), compiled from the
reference's sources and driven with its `adaptive_sampling` host code
restated in oracle/ref_cuda.py, start from the same state as this library
and are compared substep by substep.

`merge_mark_gpu` races (its compare-and-swaps decide who merges with whom)
and `split_gpu` appends children in atomicAdd order, so the deterministic
checks use scenes where the reference's outcome cannot depend on timing:
pairs of light particles that are each other's only possible partner, and
isolated heavy particles that split once each (compared as sets for the
substep of the split; the next grid sort fixes the order).  No contact
touches either scene (no gravity in the first, spacing above the contact
distance in both), so the racy contact sweep has nothing to race on.
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


def _desc(pos, gravity=(0.0, -9.81, 0.0)):
    desc = workloads.box_drop(n_side=2, substeps=4, iters=5, adaptive=1, upsample_per=0, skip=True)
    desc["particles"] = np.ascontiguousarray(pos, np.float32)
    desc["n_particles"] = pos.shape[0]
    desc["boundary"] = np.zeros((0, 3), np.float32)
    desc["n_boundary"] = 0
    desc["gravity"] = tuple(gravity)
    desc["params"].math_mode = 0  # CUDA's own cbrtf/norm3df, the functions the reference calls
    desc["params"].mass_ledger = 0  # float masses, as the reference
    return desc


def _pair(kernels, desc, masses, vel):
    s = gg.GranularSystem(**workloads.system_kwargs(desc), masses=masses, device=0)
    s.write(gg.FIELD_VEL, vel)
    refs = {}
    for fma, k in kernels.items():
        r = ref_cuda.RefSystem(k, s.read(gg.FIELD_POS), s.read(gg.FIELD_VEL), s.read(gg.FIELD_MASS),
                               np.zeros((0, 3), np.float32), cell_size=desc["cell_size"],
                               cell_length=desc["cell_length"], dt=desc["dt"], gravity=desc["gravity"],
                               density=desc["density"], max_iter=desc["params"].iters,
                               stab_iters=desc["params"].stab_iters, adaptive=True,
                               max_mass=desc["params"].max_mass)
        r.set_adaptive_last_step(s.read(gg.FIELD_ADAPTIVE_LAST_STEP))
        r.set_solver_buffers(s.read(gg.FIELD_REMOVE), s.read(gg.FIELD_MERGE), s.read(gg.FIELD_MERGE_COUNT),
                             s.read(gg.FIELD_MERGE_VELOCITY))
        refs[fma] = r
    return s, refs


FIELDS = {"pos": gg.FIELD_POS, "vel": gg.FIELD_VEL, "mass": gg.FIELD_MASS, "remove": gg.FIELD_REMOVE,
          "merge": gg.FIELD_MERGE, "merge_count": gg.FIELD_MERGE_COUNT, "als": gg.FIELD_ADAPTIVE_LAST_STEP}


def _ours(s):
    out = {k: s.read(f) for k, f in FIELDS.items()}
    out["merge_vel"] = s.read(gg.FIELD_MERGE_VELOCITY)
    return out


def _theirs(r):
    out = {k: r.read(k) for k in FIELDS}
    out["merge_vel"] = r.read("merge_vel")
    return out


def _rows(d, keys=("pos", "vel", "mass", "remove", "merge", "merge_count", "als")):
    """Rows of the per-particle fields, sorted, for comparisons as sets."""
    cols = [np.asarray(d[k], np.float64).reshape(len(d["mass"]), -1) for k in keys]
    m = np.concatenate(cols, 1)
    return m[np.lexsort(m.T[::-1])]


def _assert_equal(ours, theirs, step, as_set=False):
    n = len(ours["mass"])
    assert len(theirs["mass"]) == n, f"substep {step}: {n} particles here, {len(theirs['mass'])} in the reference"
    if as_set:
        assert np.array_equal(_rows(ours), _rows(theirs)), f"substep {step}: particle sets differ"
        return
    for k in FIELDS:
        a, b = np.asarray(ours[k]), np.asarray(theirs[k])
        assert a.shape == b.shape, (k, a.shape, b.shape)
        bad = int((a != b).reshape(n, -1).any(1).sum())
        assert bad == 0, f"substep {step}: {k} differs for {bad} particles"
    # merge_velocity is never permuted or compacted: compare the slots both keep
    m = min(len(ours["merge_vel"]), len(theirs["merge_vel"]), n)
    assert np.array_equal(ours["merge_vel"][:m], theirs["merge_vel"][:m]), f"substep {step}: merge_velocity"


MAX_MASS_PAIRS = 2.5  # the merge and split kernels' max_mass argument in the pairs scene


def _light_pairs_scene(seed=3):
    """A 14^3 lattice of heavy particles (mass 2) at spacing 0.033 with 8
    pairs of light ones (mass 1) on neighbouring sites deep inside, merged
    up to mass 2.5: a light particle's only partner with m_i + m_j <= 2.5
    within the merge radius 0.035 is its pair, heavy ones have none and
    are too light to split (mass > 2), and no two particles touch (0.033
    less the jitter stays above 2 x 0.0126 while the pairs blend)."""
    n = 14
    sp = 0.033
    p = workloads.lattice((n, n, n), sp, (0.285, 0.285, 0.285), 0.0005, seed).reshape(n, n, n, 3)
    m = np.full((n, n, n), 2.0, np.float32)
    for x0 in (4, 8):
        for y in (4, 8):
            for z in (4, 8):
                m[x0, y, z] = m[x0 + 1, y, z] = 1.0
    return p.reshape(-1, 3), m.reshape(-1)


def test_merge_marking_and_blending_match_reference_kernels(kernels):
    """(iii) merge_mark_gpu without contention, then (i) 40 substeps of
    merge_count_gpu blending with float masses, the givers' removal and the
    compaction: bit-exact against the -fmad=false build, positions within
    1e-5 r of the reference's own build, every substep."""
    pos, masses = _light_pairs_scene()
    desc = _desc(pos, gravity=(0.0, 0.0, 0.0))
    desc["params"].max_mass = MAX_MASS_PAIRS
    vel = np.tile(np.array([[0.02, 0.0, 0.0]], np.float32), (pos.shape[0], 1))
    s, refs = _pair(kernels, desc, masses, vel)
    marked = None
    for step in range(1, 46):
        s.step(1)
        for r in refs.values():
            r.step()
        ours = _ours(s)
        _assert_equal(ours, _theirs(refs[False]), step)
        e = float(np.abs(ours["pos"].astype(np.float64) - refs[True].read("pos")).max())
        assert e <= TOL, f"substep {step}: positions vs the reference's own build: {e:.3g}"
        if step == 2:
            marked = int((ours["remove"] == -1).sum())
            assert marked == 16  # 8 pairs, giver and receiver
            assert int((ours["merge"] > 0).sum()) == 8 and int((ours["merge"] < 0).sum()) == 8
    assert s.size() == pos.shape[0] - 8  # the givers left at substep 41
    assert [x[0] for x in refs[False].stats].count(8) == 1
    m = s.read(gg.FIELD_MASS)
    assert int((np.abs(m - 2.0) < 1e-3).sum()) == pos.shape[0] - 8  # heavy ones and the 8 receivers
    s.close()


def test_split_matches_reference_kernels(kernels):
    """(ii) split_gpu, check_neighborhood and extract_split_particles_kernel
    on isolated heavy surface particles (mass 4): each splits once, its
    child placed at the centre of the first empty neighbour cell.  The
    substep of the split is compared as a set (the reference appends in
    atomicAdd order), the following ones slot by slot."""
    n = 5
    pos = workloads.lattice((n, n, n), 0.15, (0.2, 0.3, 0.2), 0.005, 7)
    desc = _desc(pos)
    masses = np.full(pos.shape[0], 4.0, np.float32)
    s, refs = _pair(kernels, desc, masses, np.zeros_like(pos))
    for step in range(1, 6):
        s.step(1)
        for r in refs.values():
            r.step()
        ours = _ours(s)
        _assert_equal(ours, _theirs(refs[False]), step, as_set=(step == 1))
        e = float(np.abs(np.sort(ours["pos"], 0).astype(np.float64) - np.sort(refs[True].read("pos"), 0)).max())
        assert e <= TOL, f"substep {step}: positions vs the reference's own build: {e:.3g}"
        if step == 1:
            assert s.size() == 2 * pos.shape[0]
            assert refs[False].stats[-1][1] == pos.shape[0]
            assert np.all(ours["mass"] == 2.0)
    s.close()


def _contended_lattice(side, seed=11):
    """side^3 unit masses at spacing 2.2 r (no contact, 26 neighbours within
    the surface radius): most interior particles propose to a neighbour that
    proposes too, so the reference's compare-and-swaps race."""
    pos = workloads.lattice((side,) * 3, 0.022, (0.07, 0.07, 0.07), 0.0005, seed)
    return _desc(pos, gravity=(0.0, 0.0, 0.0))


@pytest.mark.parametrize("side", [24, 40])
def test_contended_merge_count_near_reference_runs(kernels, side):
    """(iv) Where merge_mark_gpu races, the pairs merged by this library's
    fixed schedule (merge_cas_lag = 4) against six runs of the reference's
    own kernel from the same state: measured 904 against 995-1067 (24^3)
    and 7,876 against 7,307-7,499 (40^3).  The bound is 20 % of the
    reference's mean; the phase-ordered schedule of earlier builds merged
    none."""
    desc = _contended_lattice(side)
    n = desc["n_particles"]
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    p0, v0, m0 = s.read(gg.FIELD_POS), s.read(gg.FIELD_VEL), s.read(gg.FIELD_MASS)
    s.step(2)
    ours = int((s.read(gg.FIELD_MERGE) > 0).sum())
    s.close()
    theirs = []
    for _ in range(6):
        r = ref_cuda.RefSystem(kernels[True], p0, v0, m0, np.zeros((0, 3), np.float32),
                               cell_size=desc["cell_size"], cell_length=desc["cell_length"], dt=desc["dt"],
                               gravity=desc["gravity"], density=desc["density"], adaptive=True, max_mass=4.0)
        r.step()
        r.step()
        theirs.append(int((r.read("merge") > 0).sum()))
    mean = float(np.mean(theirs))
    print(f"{side}^3: this library {ours} pairs, the reference {theirs}")
    assert mean > 0.05 * n
    assert abs(ours - mean) <= 0.2 * mean, (ours, theirs)
