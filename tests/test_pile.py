"""The adaptive-pile configuration (needs a GPU): a block on the floor and
on a 30 degree ramp of wall particles, merge/split up to mass 8 on the
integer ledger, 4 render points per particle."""
import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import abi, workloads
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def test_block_on_the_ramp_matches_oracle():
    # a block dropped onto the ramp (its surface is 0.18 high at x = 1.3)
    desc = workloads.adaptive_pile(counts=(10, 10, 10), origin=(1.25, 0.26, 0.45))
    desc["params"].math_mode = 1
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    o = orc.OracleSystem(desc)
    for k in range(60):
        s.step(1)
        o.step(1)
        assert s.size() == o.size(), k
        assert np.array_equal(s.read(gg.FIELD_POS), o.read(abi.FIELD_POS)), f"step {k}"
        assert np.array_equal(s.read(gg.FIELD_MASS_UNITS), o.read(abi.FIELD_MASS_UNITS)), f"step {k}"
    assert np.array_equal(s.read(gg.FIELD_POS, gg.SET_UPSAMPLED), o.read(abi.FIELD_POS, abi.SET_UPSAMPLED))
    # the block reached the ramp and rests on it
    p = s.read(gg.FIELD_POS)
    ramp_y = 0.005 + (p[:, 0] - 1.0) * np.tan(np.radians(30.0))
    above = (p[:, 1] > ramp_y).mean()
    print(f"fraction above the ramp after 60 substeps: {above:.3f}")
    assert above == 1.0 and np.isfinite(p).all(), above
    assert (s.read(gg.FIELD_CONTACTS) > 0).any()
    s.close()
    o.close()


def test_pile_conserves_mass_and_merges():
    desc = workloads.adaptive_pile(counts=(24, 24, 24))
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    units0 = s.stats()["total_mass_units"]
    for _ in range(300):
        s.step(1)
    st = s.stats()
    assert st["total_mass_units"] == units0 == desc["n_particles"] * abi.UNITS_PER_MASS
    assert st["merged_total"] > 0
    print(f"merged {st['merged_total']}, split {st['split_total']}, left the box through the floor "
          f"{int((s.read(gg.FIELD_POS)[:, 1] < 0).sum())} of {s.size()}")
    assert st["nonfinite"] == 0
    p = s.read(gg.FIELD_POS)
    assert np.isfinite(p).all() and (p[:, 1] > 0.005).all(), "no particle may pass through the floor"
    m = s.read(gg.FIELD_MASS)
    assert m.max() <= 8.0 and s.size() < desc["n_particles"]
    s.close()


def test_autotune_with_merge_split_restores_the_state():
    # the tuner runs trial substeps (merges and splits included) from a saved
    # copy and leaves the system as it was; every choice gives the same bits
    descs = [workloads.adaptive_pile(counts=(24, 24, 24)) for _ in range(2)]
    a, b = [gg.GranularSystem(**workloads.system_kwargs(d), device=0) for d in descs]
    a.step(30)
    b.step(30)
    st0 = b.stats()
    t = b.autotune(2)
    print("pile autotune:", t)
    assert t["trials"] == 10 and t["sweep_variant"] in (0, 1)
    st1 = b.stats()
    for k in ("n_particles", "steps", "merged_total", "split_total", "total_mass_units"):
        assert st1[k] == st0[k], k
    assert np.array_equal(a.read(gg.FIELD_POS), b.read(gg.FIELD_POS))
    for k in range(10):
        a.step(1)
        b.step(1)
        assert a.size() == b.size(), k
        assert np.array_equal(a.read(gg.FIELD_POS), b.read(gg.FIELD_POS)), k
    assert np.array_equal(a.read(gg.FIELD_MASS_UNITS), b.read(gg.FIELD_MASS_UNITS))
    a.close()
    b.close()
