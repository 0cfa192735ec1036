"""The reference's frame writers (main.cu:190-694) restated in numpy
(TEST INFRASTRUCTURE ONLY): the text each writes for given points, with the
reference's float32 centring (sums in point order) and its default stream
formatting of floats (printf "%g")."""
import numpy as np


def _g(x) -> str:
    return "%g" % float(x)


def vtk_text(title: str, pts) -> str:
    """The ASCII VTK body every writer emits, points written "x z y"."""
    pts = np.asarray(pts, np.float32).reshape(-1, 3)
    n = pts.shape[0]
    lines = ["# vtk DataFile Version 3.0", title, "ASCII", "DATASET UNSTRUCTURED_GRID", f"POINTS {n} float"]
    lines += [f"{_g(p[0])} {_g(p[2])} {_g(p[1])}" for p in pts]
    lines += [f"CELLS {n} {2 * n}"] + [f"1 {i}" for i in range(n)] + [f"CELL_TYPES {n}"] + ["1"] * n
    return "\n".join(lines) + "\n"


def valid(pts):
    pts = np.asarray(pts, np.float32).reshape(-1, 3)
    return pts[~np.isnan(pts).any(1)]


def centring(pts, divide_when_empty=True):
    """(centroid, y_offset) as main.cu:286-309 computes them."""
    f = np.float32
    pts = np.asarray(pts, f).reshape(-1, 3)
    c = np.zeros(3, f)
    if pts.shape[0]:
        c = np.array([np.add.accumulate(pts[:, k], dtype=f)[-1] for k in range(3)], f)
    if pts.shape[0] or divide_when_empty:
        with np.errstate(invalid="ignore", divide="ignore"):
            c = c / f(pts.shape[0])
    min_y = f(1000000.0)
    if pts.shape[0]:
        min_y = min(min_y, np.min(pts[:, 1] - c[1]))
    return c, (f(-min_y) if min_y < 0 else f(0))


def centre(pts, c, y_offset):
    f = np.float32
    pts = np.asarray(pts, f).reshape(-1, 3)
    return np.stack([pts[:, 0] - c[0], (pts[:, 1] - c[1]) + f(y_offset), pts[:, 2] - c[2]], 1).astype(f)


def by_mass(pos, mass):
    """saveParticlesByMass: {"light" | "medium" | "heavy": text} for the
    non-empty groups."""
    pos = np.asarray(pos, np.float32).reshape(-1, 3)
    mass = np.asarray(mass, np.float32)
    ok = ~np.isnan(pos).any(1)
    c, y0 = centring(pos[ok], divide_when_empty=False)
    cp = centre(pos[ok], c, y0)
    m = mass[ok]
    groups = {"light": m < 2, "medium": (m >= 2) & (m <= 3)}
    groups["heavy"] = ~(groups["light"] | groups["medium"])
    return {k: vtk_text("Particles by Mass", cp[sel]) for k, sel in groups.items() if sel.any()}


def csv_text(pts) -> str:
    pts = np.asarray(pts, np.float32).reshape(-1, 3)
    return "".join(f"{_g(p[0])},{_g(p[1])},{_g(p[2])}\n" for p in pts)
