"""Whole-substep parity at the benchmark sizes, through the C ABI.

The 8,388,608-particle column collapse (248 x 124 x 124 cells, 22-bit keys,
three radix passes, 33,554,432 render points) and the 262,144-particle
adaptive pile, stepped by the library in math mode 1 and by the FP32 oracle
from the same scene: keys, sorted order, cell table, positions,
velocities, masses, the merge/split bookkeeping and the render points must
be bit-identical.

The merge scan takes its local density from the surface pass when the
surface pass's search radius 2.0002 (r_i + r_max) covers the merge radius,
and sums it itself otherwise.  With the reference's merge radius 0.035 both
scenes here take the second path (r = 0.002 and 0.005); the column with
lengths scaled by r / 0.01 and the box drops of test_gpu_parity.py
(r = 0.01) take the first.
"""
import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import abi, workloads
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def _pair(desc):
    desc["params"].math_mode = 1
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    o = orc.OracleSystem(desc, fp64=False)
    return s, o


def _same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, f"{what}: shapes {a.shape} vs {b.shape}"
    bad = (a != b).reshape(a.shape[0], -1).any(1) if a.ndim else a != b
    nb = int(np.count_nonzero(bad))
    assert nb == 0, f"{what}: {nb} entries differ, first at {np.nonzero(bad)[0][:5]}"


def _compare_all(s, o, step, upsampled=True):
    assert s.size() == o.size(), f"substep {step}: {s.size()} vs {o.size()} particles"
    for f in (gg.FIELD_CELL_KEY, gg.FIELD_PERM, gg.FIELD_CELL_START, gg.FIELD_POS, gg.FIELD_VEL, gg.FIELD_MASS,
              gg.FIELD_MASS_UNITS, gg.FIELD_SURFACE, gg.FIELD_REMOVE, gg.FIELD_MERGE_COUNT,
              gg.FIELD_NUM_CONSTRAINTS):
        _same(s.read(f), o.read(f), f"substep {step}: field {f}")
    if upsampled:
        _same(s.read(gg.FIELD_POS, gg.SET_UPSAMPLED), o.read(abi.FIELD_POS, abi.SET_UPSAMPLED),
              f"substep {step}: render-point positions")
        _same(s.read(gg.FIELD_VEL, gg.SET_UPSAMPLED), o.read(abi.FIELD_VEL, abi.SET_UPSAMPLED),
              f"substep {step}: render-point velocities")


def _surface_pass_covers_merge_radius(desc):
    """The library's condition for taking the merge density from the
    surface pass, for unit masses (r_max = r)."""
    r = float(np.cbrt(3.0 / (4.0 * np.pi * desc["density"])))
    return desc["params"].merge_radius * 1.0001 <= 2.0002 * (r + r)


@pytest.mark.parametrize("constants", ["reference", "scaled"])
def test_column_8m_substeps_match_oracle(constants):
    desc = workloads.column_collapse(counts=(128, 256, 256), constants=constants)
    assert desc["n_particles"] == 8_388_608 and desc["n_upsampled"] == 33_554_432
    assert int(np.prod(desc["cell_size"])) == 248 * 124 * 124
    assert _surface_pass_covers_merge_radius(desc) == (constants == "scaled")
    s, o = _pair(desc)
    _compare_all(s, o, 1)  # the constructor's substep
    s.step(1)
    o.step(1)
    _compare_all(s, o, 2)  # the first merge marking
    st = s.stats()
    assert st["total_mass_units"] == desc["n_particles"] * abi.UNITS_PER_MASS
    s.close()
    o.close()


def test_adaptive_pile_262k_through_its_first_merges():
    desc = workloads.adaptive_pile()
    assert desc["n_particles"] == 262_144
    assert not _surface_pass_covers_merge_radius(desc)
    s, o = _pair(desc)
    marked = 0
    for step in range(2, 47):
        s.step(1)
        o.step(1)
        marked = max(marked, int((s.read(gg.FIELD_REMOVE) == -1).sum()))
        if step % 5 == 0 or step >= 40:
            _compare_all(s, o, step)
    st = s.stats()
    assert marked > 0, "the pile must start merges"
    assert st["total_mass_units"] == desc["n_particles"] * abi.UNITS_PER_MASS
    s.close()
    o.close()
