"""The learned warm start inside the substep (needs a GPU): the recording
mode's features and targets, the residual mode, the switch-off path and
what the trained network (granular_gpu_gb300/weights) gains over the plain
solver on held-out scenes."""
import os

import numpy as np
import pytest

import granular_gpu_gb300 as gg
from granular_gpu_gb300 import learn as L, workloads

pytestmark = pytest.mark.gpu


def _system(desc, mlp=None, attach=False):
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    if attach or mlp is not None:
        s.set_warm_start(mlp)
    return s


def test_record_mode_features_and_targets():
    desc = L.pile_scene(3, dims=(0.15, 0.15, 0.15), drop=0.0, target_residual=1e-2 * L.R)
    desc["params"].warm_start = 2
    s = _system(desc, attach=True)
    s.step(20)  # landed
    x0, v0 = s.read(gg.FIELD_POS), s.read(gg.FIELD_VEL)
    s.step(1)
    perm = s.read(gg.FIELD_PERM)
    dt = np.float32(desc["dt"])
    g = np.array(desc["gravity"], np.float32)
    dv = dt * g
    xs0 = x0[perm] + dt * (v0[perm] + dv)
    slen = np.float32(np.linalg.norm(g.astype(np.float64)) * float(dt) ** 2)
    want = (s.read(gg.FIELD_POS) - xs0) / slen
    got = s.read(gg.FIELD_WARM_TARGET)
    assert np.abs(got - want).max() <= 1e-3 * (np.abs(want).max() + 1.0)
    assert np.abs(want).max() > 0.5, "the sweeps must move the particles"
    feat = s.read(gg.FIELD_FEATURES)
    assert feat.shape == (s.size(), 48)
    f = (feat.astype(np.uint32) << 16).view(np.float32)
    assert np.all(f[:, 0] == 1.0) and np.all(f[:, 7] == 1.0)  # bias input, unit masses
    assert (f[:, 9] > 0).any(), "contacts must appear in the features"
    s.close()


def test_residual_mode_stops_at_tolerance_or_cap():
    tol = 1e-2 * L.R
    desc = L.pile_scene(4, dims=(0.2, 0.2, 0.2), drop=0.0, target_residual=tol, max_sweeps=60)
    s = _system(desc)
    for _ in range(30):
        s.step(1)
        st = s.stats()
        assert st["last_sweeps"] <= 60
        assert st["last_residual"] <= tol or st["last_sweeps"] == 60
        assert st["last_residual_max"] >= st["last_residual"]
    s.close()


def test_switched_off_warm_start_changes_nothing():
    desc = L.pile_scene(5, dims=(0.15, 0.15, 0.15), drop=0.01)
    desc["params"].target_residual = 0.0  # the reference's fixed sweeps
    a = _system(desc)
    m = gg.Mlp(seed=9)
    b = _system(desc, mlp=m)  # attached, warm_start = 0
    a.step(25)
    b.step(25)
    assert np.array_equal(a.read(gg.FIELD_POS), b.read(gg.FIELD_POS))
    assert np.array_equal(a.read(gg.FIELD_VEL), b.read(gg.FIELD_VEL))
    a.close()
    b.close()
    m.close()


@pytest.mark.skipif(not os.path.exists(L.WEIGHTS), reason="trained weights not present")
def test_trained_network_gains_over_plain_solver():
    m = L.load_mlp()
    res = L.evaluate(m, seeds=(103,), frames=80, dims=(0.35, 0.3, 0.35))
    print(res)
    assert res["sweep_ratio"] <= 0.6, res
    assert res["time_ratio"] <= 0.75, res
    m.close()
