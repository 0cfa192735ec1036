"""Scene descriptions of the configurations (CPU only): the analytic walls of
the configured mode sit where the wall particles are, and the configured
parameters are the ones the configurations state."""
import math

import numpy as np

from granular_gpu_gb300 import workloads


def _planes(params):
    return [(np.array(list(params.planes[k])[:3]), params.planes[k][3]) for k in range(params.n_planes)]


def test_box_planes_lie_on_the_wall_particles():
    space = (2.0, 1.0, 1.0)
    L = np.float32(workloads.CELL_PER_RADIUS * 0.002)
    walls, _ = workloads.box_walls(space, L)
    for n, d in workloads.box_planes(space):
        s = walls.astype(np.float64) @ n - d
        assert s.min() > -1e-6  # every wall particle on or inside the half-space
        assert np.isclose(s.min(), 0.0, atol=1e-6)  # and the face's particles on the plane


def test_ramp_plane_matches_the_ramp_walls():
    space = (2.0, 1.0, 1.0)
    L = np.float32(workloads.CELL_PER_RADIUS * 0.005)
    ramp = workloads.ramp_walls(space, L, 30.0).astype(np.float64)
    n, d = workloads.ramp_plane(space, 30.0)
    assert np.isclose(np.linalg.norm(n), 1.0)
    assert np.abs(ramp @ n - d).max() < 1e-5  # the wall particles lie on the plane
    floor = 0.005 * space[1]
    assert np.array([0.2, floor + 1e-3, 0.5]) @ n - d > 0  # before the ramp the floor binds, not the plane
    assert math.isclose(math.degrees(math.atan2(-n[0], n[1])), 30.0, abs_tol=1e-9)


def test_configured_parameters_follow_the_configurations():
    box = workloads.box_drop(n_side=8, substeps=4, iters=3, configured=True)["params"]
    assert (box.contact_law, box.split_claim, box.stab_iters, box.iters) == (1, 1, 0, 3)
    assert np.isclose(box.mu_static, 0.5) and np.isclose(box.mu_kinetic, 0.4) and box.n_planes == 6
    pile = workloads.adaptive_pile(counts=(4, 4, 4), configured=True)["params"]
    assert pile.n_planes == 7  # the box faces and the 30-degree ramp
    col = workloads.column_collapse(counts=(4, 8, 8), constants="configured")["params"]
    assert col.contact_law == 1 and col.n_planes == 6 and col.merge_enabled == 1
    ref = workloads.column_collapse(counts=(4, 8, 8), constants="reference")["params"]
    assert ref.contact_law == 0 and ref.n_planes == 0 and ref.split_claim == 0
