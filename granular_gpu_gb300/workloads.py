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


def set_planes(params, planes):
    """Analytic walls (n, d): a particle keeps n . x >= d + r.  Normals are
    normalised here."""
    params.n_planes = len(planes)
    for k, (n, d) in enumerate(planes):
        n = np.asarray(n, np.float64)
        n = n / np.linalg.norm(n)
        for c in range(3):
            params.planes[k][c] = float(n[c])
        params.planes[k][3] = float(d)
    return params


def box_planes(space_size, inset=0.005):
    """The six faces of the box, where the wall particles of box_walls lie
    (inset by 0.5 % of each side), as analytic walls."""
    sp = np.asarray(space_size, np.float64)
    out = []
    for a in range(3):
        n = np.zeros(3)
        n[a] = 1.0
        out.append((n.copy(), inset * sp[a]))
        out.append((-n, -(1.0 - inset) * sp[a]))
    return out


def configure(params, mu_static=0.5, mu_kinetic=0.4, planes=()):
    """Configured mode: Coulomb friction mu_static / mu_kinetic (restitution
    0), children that claim their cell, and analytic walls.  The scene's
    Jacobi sweeps are all the solver runs (no stabilisation sweeps, which
    move the substep's start positions and let resting contacts creep)."""
    params.contact_law = 1
    params.stab_iters = 0
    params.mu_static, params.mu_kinetic = float(mu_static), float(mu_kinetic)
    params.split_claim = 1
    return set_planes(params, list(planes))


def _desc(particles, walls, upsampled, space, L, cs, dt, g, density, adaptive, params, skip=False):
    return dict(particles=particles, n_particles=particles.shape[0], boundary=walls,
                n_boundary=walls.shape[0], upsampled=upsampled,
                n_upsampled=0 if upsampled is None else upsampled.shape[0],
                space_size=tuple(space), cell_length=float(L), dt=float(dt), gravity=tuple(g),
                cell_size=tuple(cs), density=float(density), upsampled_radius=0.005,
                is_move_boundary=0, is_adaptive=int(adaptive), skip_initial_step=int(skip),
                device=0, max_particles=0, params=params)


def box_drop(n_side=32, seed=42, substeps=4, iters=3, adaptive=0, upsample_per=0, skip=False, configured=False):
    """Plain PBD box drop: n_side^3 unit masses, r = 0.01, lattice spacing 2r
    with uniform jitter +-0.05r, block centred 0.5 above the floor of a 1^3
    box, dt = 1/60 split into `substeps`, `iters` Jacobi sweeps.
    configured=True: the configuration's contact model (Coulomb friction
    0.5 / 0.4, restitution 0, the box faces as analytic walls)."""
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
    if configured:
        configure(params, 0.5, 0.4, box_planes(space))
    ups = None
    if upsample_per:
        rng = np.random.default_rng(seed + 1)
        ups = (np.repeat(p, upsample_per, 0) + rng.uniform(-r, r, (p.shape[0] * upsample_per, 3))).astype(np.float32)
    return _desc(p, walls, ups, space, L, cs, dt, (0.0, -9.81, 0.0), REF_DENSITY, adaptive, params, skip)


def column_collapse(counts=(128, 256, 256), r=0.002, seed=42, substeps=4, iters=4, upsample_per=4,
                    adaptive=1, skip=False, constants="scaled"):
    """Column collapse: counts lattice (x, y, z) of unit masses of radius r
    at spacing 1.925r (the 2x1x1 box cannot hold 2^23 spheres at 2r with
    aspect 2), jitter +-0.05r, resting in the -x end of a 2x1x1 box;
    dt = 1/120 split into `substeps`; merge/split up to mass 8 on the exact
    integer ledger; `upsample_per` render points per particle.

    constants="scaled" scales every length constant of the reference by
    r / 0.01 and advects render points with the substep's dt;
    constants="configured" adds the configured mode to that (Coulomb
    friction 0.5 / 0.4, claiming split children, the box faces as analytic
    walls);
    constants="reference" keeps them as compiled into the reference's
    kernels (wall reach 0.01 + max(r, 0.01), merge radius 0.035, upsampling
    support 0.045 and step 0.002, ...), as the reference's own build runs
    this scene."""
    L = np.float32(CELL_PER_RADIUS * r)
    space = (2.0, 1.0, 1.0)
    walls, cs = box_walls(space, L)
    s = 1.925 * r
    o = 0.0095 * (r / 0.002)
    p = lattice(counts, s, (o, o, o), 0.05 * r, seed)
    dt = 1.0 / 120.0 / substeps
    if constants == "reference":
        params = scaled_params(REF_RADIUS, iters=iters, dt_sub=None, max_mass=8.0, ledger=1)
    elif constants in ("scaled", "configured"):
        params = scaled_params(r, iters=iters, dt_sub=dt, max_mass=8.0, ledger=1)
        if constants == "configured":
            # the configuration's contact model: Coulomb friction 0.5 / 0.4,
            # restitution 0, split children that claim their cell, and the
            # box faces as analytic walls behind the wall particles
            configure(params, 0.5, 0.4, box_planes(space))
    else:
        raise ValueError(constants)
    params.merge_enabled = 1 if adaptive else 0
    params.upsample_enabled = 1 if upsample_per else 0
    ups = None
    if upsample_per:
        rng = np.random.default_rng(seed + 1)
        ups = (np.repeat(p, upsample_per, 0) + rng.uniform(-r, r, (p.shape[0] * upsample_per, 3))).astype(np.float32)
    return _desc(p, walls, ups, space, L, cs, dt, (0.0, -9.81, 0.0), density_for_radius(r), adaptive, params,
                 skip)


def ramp_walls(space_size, cell_length, angle_deg=30.0, x0=None, x1=None):
    """Wall particles of an inclined plane across the box (z fills the box):
    a lattice as fine as the box walls (half a cell), rising at `angle_deg`
    from the floor at x0 (default: half the box) to x1 (default: the far
    wall).  The reference builds every obstacle from wall particles
    (main.cu:849-1167), so a ramp is one more particle set."""
    sp = np.asarray(space_size, np.float64)
    h = float(cell_length) / 2.0
    floor = 0.005 * sp[1]
    x0 = 0.5 * sp[0] if x0 is None else x0
    x1 = 0.995 * sp[0] if x1 is None else x1
    t = math.tan(math.radians(angle_deg))
    length = (x1 - x0) / math.cos(math.radians(angle_deg))
    nu = max(2, int(math.ceil(length / h)) + 1)
    nz = max(2, int(math.ceil(0.99 * sp[2] / h)) + 1)
    u = np.linspace(0.0, x1 - x0, nu)
    z = np.linspace(0.005 * sp[2], 0.995 * sp[2], nz)
    U, Z = np.meshgrid(u, z, indexing="ij")
    pts = np.stack([x0 + U, floor + U * t, Z], -1).reshape(-1, 3)
    keep = pts[:, 1] <= 0.995 * sp[1]
    return pts[keep].astype(np.float32)


def adaptive_pile(counts=(64, 64, 64), r=0.005, seed=42, substeps=1, iters=5, upsample_per=4, ledger=1,
                  max_mass=8.0, origin=None, scaled=False, configured=False):
    """The adaptive-pile configuration: fine particles of radius r in a
    jittered block at spacing 2r (64^3 = 262,144 particles fill a 0.64 m
    block: the 0.6 x 0.4 x 0.6 m block of the configuration holds only
    144,000 at that spacing), released 0.02 above the floor of a 2 x 1 x 1
    box at its -x end, with a 30 degree ramp of wall particles over the +x
    half; merge/split up to mass `max_mass` (levels 1/2/4/8) on the integer
    ledger; `upsample_per` render points per particle; dt = 1/240.

    The reference's length constants (wall reach 0.01 + max(r, 0.01), merge
    radius 0.035, upsampling support 0.045, ...) are kept as compiled in,
    as the reference would run this scene (`scaled=True` scales them by
    r / 0.01 instead).  Scaled, the wall reach drops to 2r while the wall
    particles stay half a cell apart, and a pile this tall presses most
    particles through the one-particle-thick floor.

    configured=True adds the configured mode: Coulomb friction 0.5 / 0.4,
    claiming split children, and the box faces and the ramp as analytic
    walls behind their wall particles."""
    L = np.float32(CELL_PER_RADIUS * r)
    space = (2.0, 1.0, 1.0)
    walls, cs = box_walls(space, L)
    walls = np.concatenate([walls, ramp_walls(space, L, 30.0)]).astype(np.float32)
    floor = 0.005 * space[1]
    if origin is None:
        origin = (0.05, floor + 0.01 * (r / 0.01) + r + 0.02, 0.5 - (counts[2] - 1) * r)
    p = lattice(counts, 2 * r, origin, 0.05 * r, seed)
    dt = 1.0 / 240.0 / substeps
    params = scaled_params(r if scaled else REF_RADIUS, iters=iters, dt_sub=None, max_mass=max_mass, ledger=ledger)
    params.upsample_enabled = 1 if upsample_per else 0
    params.merge_enabled = 1
    if configured:
        configure(params, 0.5, 0.4, box_planes(space) + [ramp_plane(space, 30.0)])
    ups = None
    if upsample_per:
        rng = np.random.default_rng(seed + 1)
        ups = (np.repeat(p, upsample_per, 0) + rng.uniform(-r, r, (p.shape[0] * upsample_per, 3))).astype(np.float32)
    return _desc(p, walls, ups, space, L, cs, dt, (0.0, -9.81, 0.0), density_for_radius(r), 1, params)


def ramp_plane(space_size, angle_deg=30.0, x0=None):
    """The ramp of ramp_walls as an analytic wall: y >= floor + tan(angle)
    (x - x0).  Below x0 the half-space lies under the floor, so it binds
    only over the ramp."""
    sp = np.asarray(space_size, np.float64)
    floor = 0.005 * sp[1]
    x0 = 0.5 * sp[0] if x0 is None else x0
    a = math.radians(angle_deg)
    n = np.array([-math.sin(a), math.cos(a), 0.0])
    return (n, float(n @ np.array([x0, floor, 0.0])))


def system_kwargs(desc: dict) -> dict:
    """Keyword arguments of GranularSystem(...) from a workload dict."""
    return dict(particles=desc["particles"], boundary_particles=desc["boundary"],
                upsampled_particles=desc["upsampled"], space_size=desc["space_size"],
                cell_length=desc["cell_length"], dt=desc["dt"], g=desc["gravity"],
                cell_size=desc["cell_size"], density=desc["density"],
                upsampled_radius=desc["upsampled_radius"], is_move_boundary=desc["is_move_boundary"],
                is_adaptive=desc["is_adaptive"], params=desc["params"],
                skip_initial_step=bool(desc["skip_initial_step"]), max_particles=desc["max_particles"])
