"""Synthetic scenes for the benchmark configurations.

The reference ships no benchmark inputs; these generators build seeded
lattices with the shapes, sizes and distributions the benchmark
configurations name, plus the reference's box walls (main.cu:849-888).
Each returns keyword arguments for GranularSystem(...) and for the oracle.
"""
import math

import numpy as np

from . import abi

REF_RADIUS = 0.01             # radius of a unit mass at the reference density
REF_DENSITY = 238732.4146     # scenes/box.json: r = 0.01 at mass 1
CELL_PER_RADIUS = 4.04        # reference cell_length 0.0404 for r = 0.01


def density_for_radius(r: float) -> float:
    """Density giving radius r to a unit mass, rounded to an integer so the
    int and float density laws of the reference coincide."""
    return float(round(3.0 / (4.0 * math.pi * r ** 3)))


def box_walls(space_size, cell_length):
    """Wall particles of the reference's BOX scene (main.cu:849-888): six
    faces of a lattice twice as fine as the cell grid, inset by 0.5%."""
    sp = np.asarray(space_size, np.float32)
    L = np.float32(cell_length)
    cs = [int(math.ceil(np.float32(sp[i]) / L)) for i in range(3)]
    c0, c1, c2 = 2 * cs[0], 2 * cs[1], 2 * cs[2]
    den = np.array([c0 - 1, c1 - 1, c2 - 1], np.float32)

    def face(a, b, c):
        x = np.stack(np.broadcast_arrays(a, b, c), -1).reshape(-1, 3).astype(np.float32)
        x = x / den * sp
        return np.float32(0.99) * x + np.float32(0.005) * sp

    i0, j1 = np.meshgrid(np.arange(c0), np.arange(c1), indexing="ij")
    parts = [face(i0, j1, 0), face(i0, j1, c2 - 1)]
    i0, k1 = np.meshgrid(np.arange(c0), np.arange(c2 - 2) + 1, indexing="ij")
    parts += [face(i0, 0, k1), face(i0, c1 - 1, k1)]
    j1, k1 = np.meshgrid(np.arange(c1 - 2) + 1, np.arange(c2 - 2) + 1, indexing="ij")
    parts += [face(0, j1, k1), face(c0 - 1, j1, k1)]
    # (face order differs from the reference's loop order; callers pass the
    # same array to every implementation, and the sort is stable)
    walls = np.concatenate(parts, 0)
    return walls.astype(np.float32), cs


def lattice(counts, spacing, origin, jitter, seed):
    """counts[0] x counts[1] x counts[2] points, x fastest-varying last."""
    g = [np.arange(c, dtype=np.float64) for c in counts]
    X, Y, Z = np.meshgrid(*g, indexing="ij")
    p = np.stack([origin[0] + spacing * X, origin[1] + spacing * Y, origin[2] + spacing * Z], -1)
    p = p.reshape(-1, 3)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        p = p + rng.uniform(-jitter, jitter, p.shape)
    return p.astype(np.float32)


def scaled_params(r: float, iters: int, stab_iters: int = 3, dt_sub: float = None,
                  max_mass: float = 4.0, ledger: int = 0):
    """Reference constants with every length scaled by r / 0.01 (the
    reference's scenes are built for r = 0.01)."""
    s = r / REF_RADIUS
    p = abi.default_params()
    p.stab_iters, p.iters = stab_iters, iters
    p.boundary_radius = 0.01 * s
    p.boundary_min_radius = 0.01 * s
    p.merge_radius = 0.035 * s
    p.up_inv_h2 = 1.0 / (0.045 * s) ** 2
    p.up_boundary_radius = 0.015 * s
    p.up_floor_y = 0.04 * s
    p.up_ground_band = 0.1 * s
    if dt_sub is not None:
        p.up_dt = dt_sub
    p.max_mass = max_mass
    p.mass_ledger = ledger
    return p


def _desc(particles, walls, upsampled, space, L, cs, dt, g, density, adaptive, params, skip=False):
    return dict(particles=particles, n_particles=particles.shape[0], boundary=walls,
                n_boundary=walls.shape[0], upsampled=upsampled,
                n_upsampled=0 if upsampled is None else upsampled.shape[0],
                space_size=tuple(space), cell_length=float(L), dt=float(dt), gravity=tuple(g),
                cell_size=tuple(cs), density=float(density), upsampled_radius=0.005,
                is_move_boundary=0, is_adaptive=int(adaptive), skip_initial_step=int(skip),
                device=0, max_particles=0, params=params)


def box_drop(n_side=32, seed=42, substeps=4, iters=3, adaptive=0, upsample_per=0, skip=False):
    """Plain PBD box drop: n_side^3 unit masses, r = 0.01, lattice spacing 2r
    with uniform jitter +-0.05r, block centred 0.5 above the floor of a 1^3
    box, dt = 1/60 split into `substeps`, `iters` Jacobi sweeps."""
    r = REF_RADIUS
    L = np.float32(CELL_PER_RADIUS * r)
    space = (1.0, 1.0, 1.0)
    walls, cs = box_walls(space, L)
    span = (n_side - 1) * 2 * r
    origin = (0.5 - span / 2, 0.5 - span / 2, 0.5 - span / 2)
    p = lattice((n_side,) * 3, 2 * r, origin, 0.05 * r, seed)
    dt = 1.0 / 60.0 / substeps
    params = scaled_params(r, iters=iters, dt_sub=None)
    params.upsample_enabled = 1 if upsample_per else 0
    params.merge_enabled = 1 if adaptive else 0
    ups = None
    if upsample_per:
        rng = np.random.default_rng(seed + 1)
        ups = (np.repeat(p, upsample_per, 0) + rng.uniform(-r, r, (p.shape[0] * upsample_per, 3))).astype(np.float32)
    return _desc(p, walls, ups, space, L, cs, dt, (0.0, -9.81, 0.0), REF_DENSITY, adaptive, params, skip)


def column_collapse(counts=(128, 256, 256), r=0.002, seed=42, substeps=4, iters=4, upsample_per=4,
                    adaptive=1, skip=False):
    """Column collapse: counts lattice (x, y, z) of unit masses of radius r
    at spacing 1.925r (the 2x1x1 box cannot hold 2^23 spheres at 2r with
    aspect 2), jitter +-0.05r, resting in the -x end of a 2x1x1 box;
    dt = 1/120 split into `substeps`; merge/split up to mass 8 on the exact
    integer ledger; `upsample_per` render points per particle."""
    L = np.float32(CELL_PER_RADIUS * r)
    space = (2.0, 1.0, 1.0)
    walls, cs = box_walls(space, L)
    s = 1.925 * r
    o = 0.0095 * (r / 0.002)
    p = lattice(counts, s, (o, o, o), 0.05 * r, seed)
    dt = 1.0 / 120.0 / substeps
    params = scaled_params(r, iters=iters, dt_sub=dt, max_mass=8.0, ledger=1)
    params.merge_enabled = 1 if adaptive else 0
    params.upsample_enabled = 1 if upsample_per else 0
    ups = None
    if upsample_per:
        rng = np.random.default_rng(seed + 1)
        ups = (np.repeat(p, upsample_per, 0) + rng.uniform(-r, r, (p.shape[0] * upsample_per, 3))).astype(np.float32)
    return _desc(p, walls, ups, space, L, cs, dt, (0.0, -9.81, 0.0), density_for_radius(r), adaptive, params,
                 skip)


def system_kwargs(desc: dict) -> dict:
    """Keyword arguments of GranularSystem(...) from a workload dict."""
    return dict(particles=desc["particles"], boundary_particles=desc["boundary"],
                upsampled_particles=desc["upsampled"], space_size=desc["space_size"],
                cell_length=desc["cell_length"], dt=desc["dt"], g=desc["gravity"],
                cell_size=desc["cell_size"], density=desc["density"],
                upsampled_radius=desc["upsampled_radius"], is_move_boundary=desc["is_move_boundary"],
                is_adaptive=desc["is_adaptive"], params=desc["params"],
                skip_initial_step=bool(desc["skip_initial_step"]), max_particles=desc["max_particles"])
