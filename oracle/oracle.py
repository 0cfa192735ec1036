"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module.  It exposes the same create/step/read surface as the
CUDA library so parity tests read symmetrically.
"""
import ctypes as C
import os

import numpy as np

from granular_gpu_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))


def _load(fp64: bool) -> C.CDLL:
    name = "libggoracle64.so" if fp64 else "libggoracle32.so"
    path = os.path.join(HERE, "_build", name)
    if not os.path.exists(path):
        from oracle import build as _b
        _b.build()
    lib = C.CDLL(path)
    pre = "ggo64_" if fp64 else "ggo32_"
    sig = {
        "default_params": (None, [C.POINTER(abi.gg_params)]),
        "create": (C.c_void_p, [C.POINTER(abi.gg_desc)]),
        "step": (None, [C.c_void_p, C.c_int]),
        "size": (C.c_int64, [C.c_void_p, C.c_int]),
        "steps": (C.c_int64, [C.c_void_p]),
        "n_grid": (C.c_int64, [C.c_void_p]),
        "merged_last": (C.c_int64, [C.c_void_p]),
        "split_last": (C.c_int64, [C.c_void_p]),
        "read": (C.c_int64, [C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
        "write": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_int64]),
        "grid_build": (None, [C.POINTER(C.c_float), C.c_int64, C.POINTER(C.c_int32), C.c_float,
                              C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                              C.POINTER(C.c_int32)]),
        "save_particle_stats": (C.c_int, [C.c_void_p, C.c_char_p]),
        "error_word": (C.c_int32, [C.c_void_p]),
        "threads": (C.c_int, []),
        "destroy": (None, [C.c_void_p]),
        "animate_walls": (None, [C.c_void_p, C.POINTER(C.c_float), C.c_float, C.POINTER(C.c_float)]),
    }
    for k, (res, args) in sig.items():
        fn = getattr(lib, pre + k)
        fn.restype = res
        fn.argtypes = args
    lib._pre = pre
    return lib


_LIBS = {}


def lib(fp64: bool = False) -> C.CDLL:
    if fp64 not in _LIBS:
        _LIBS[fp64] = _load(fp64)
    return _LIBS[fp64]


def _fn(l, name):
    return getattr(l, l._pre + name)


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32)) if a is not None else None


def grid_build(pos, cell_size, cell_length, fp64=False):
    """keys, sorted_keys, perm, cell_start of the oracle's grid build."""
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    n = pos.shape[0]
    cs = np.ascontiguousarray(cell_size, dtype=np.int32)
    ncell = int(cs[0]) * int(cs[1]) * int(cs[2])
    keys = np.zeros(max(n, 1), np.int32)
    sk = np.zeros(max(n, 1), np.int32)
    perm = np.zeros(max(n, 1), np.int32)
    cstart = np.zeros(ncell + 1, np.int32)
    l = lib(fp64)
    _fn(l, "grid_build")(_fptr(pos), n, _iptr(cs), C.c_float(cell_length),
                         _iptr(keys), _iptr(sk), _iptr(perm), _iptr(cstart))
    return keys[:n], sk[:n], perm[:n], cstart


class OracleSystem:
    """The CPU restatement behind the same surface as the CUDA system."""

    def __init__(self, desc_fields: dict, fp64: bool = False):
        self._lib = lib(fp64)
        self._keep = []
        d = abi.gg_desc()
        for k, v in desc_fields.items():
            if k in ("particles", "boundary", "upsampled", "masses"):
                if v is None:
                    continue
                a = np.ascontiguousarray(v, dtype=np.float32)
                self._keep.append(a)
                setattr(d, k, _fptr(a))
            elif k == "boundary_animated":
                if v is None:
                    continue
                a = np.ascontiguousarray(v, dtype=np.int32)
                self._keep.append(a)
                d.boundary_animated = _iptr(a)
            elif k in ("space_size", "gravity"):
                for i in range(3):
                    getattr(d, k)[i] = float(v[i])
            elif k == "cell_size":
                for i in range(3):
                    d.cell_size[i] = int(v[i])
            elif k == "params":
                d.params = v
            else:
                setattr(d, k, v)
        self._h = _fn(self._lib, "create")(C.byref(d))
        self.cell_size = tuple(int(x) for x in desc_fields["cell_size"])

    def step(self, n: int = 1):
        _fn(self._lib, "step")(self._h, n)

    def size(self, s: int = abi.SET_GRANULAR) -> int:
        return int(_fn(self._lib, "size")(self._h, s))

    @property
    def steps(self):
        return int(_fn(self._lib, "steps")(self._h))

    def merged_last(self):
        return int(_fn(self._lib, "merged_last")(self._h))

    def split_last(self):
        return int(_fn(self._lib, "split_last")(self._h))

    def read(self, field: int, s: int = abi.SET_GRANULAR):
        dt, comp = abi.FIELD_LAYOUT[field]
        if field == abi.FIELD_CELL_START:
            n = self.cell_size[0] * self.cell_size[1] * self.cell_size[2] + 1
        elif field in (abi.FIELD_CELL_KEY, abi.FIELD_PERM) and s == abi.SET_GRANULAR:
            n = max(self.size(s), int(_fn(self._lib, "n_grid")(self._h)))
        else:
            n = self.size(s)
        out = np.zeros((max(n, 1), comp), dtype=dt)
        got = _fn(self._lib, "read")(self._h, s, field, out.ctypes.data)
        if got < 0:
            raise KeyError(f"field {field} not available for set {s}")
        out = out[:got]
        return out[:, 0] if comp == 1 else out

    def write(self, field: int, data, s: int = abi.SET_GRANULAR):
        a = np.ascontiguousarray(data, dtype=np.float32).reshape(-1, 3)
        rc = _fn(self._lib, "write")(self._h, s, field, _fptr(a), a.shape[0])
        if rc != 0:
            raise ValueError("oracle write failed")

    def animate_walls(self, translation, rotation, center):
        """animateParticles (main.cu:1175-1208) on the oracle's walls."""
        t = np.ascontiguousarray(translation, np.float32)
        c = np.ascontiguousarray(center, np.float32)
        _fn(self._lib, "animate_walls")(self._h, _fptr(t), float(np.float32(rotation)), _fptr(c))

    def save_particle_stats(self, path: str):
        _fn(self._lib, "save_particle_stats")(self._h, path.encode())

    def error_word(self) -> int:
        return int(_fn(self._lib, "error_word")(self._h))

    def close(self):
        if self._h:
            _fn(self._lib, "destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def threads() -> int:
    return int(_fn(lib(False), "threads")())


def color_dots(pos, mass=None, surface=None, sdist=None, mode=2, min_mass=1.0, max_mass=4.0):
    """generate_dots_CUDA (VBO.hpp:9-71) restated in float32 numpy: packed
    positions and colours.  mode 0: surface == 1 -> (0.34, 0.46, 0.7), else
    black; mode 1: distance == 0 -> (0.34, 0.46, 0.7), >= 100 -> black, else
    red; mode 2: (1 - t) * blue + t * red with t = (m - min) / (max - min),
    and mass == 0 -> (6.0 / 255 / 0, 214 / 255, 160 / 255), first component
    +inf.  Missing arrays read as the reference's zero-filled ones."""
    f = np.float32
    pos = np.asarray(pos, f).reshape(-1, 3)
    n = pos.shape[0]
    m = np.zeros(n, f) if mass is None else np.asarray(mass, f)
    sf = np.zeros(n, np.int32) if surface is None else np.asarray(surface, np.int32)
    sd = np.zeros(n, f) if sdist is None else np.asarray(sdist, f)
    col = np.zeros((n, 3), f)
    blue_grey = np.array([0.34, 0.46, 0.7], f)
    if mode == 0:
        col[sf == 1] = blue_grey
    elif mode == 1:
        col[sd == 0] = blue_grey
        col[(sd != 0) & ~(sd >= f(100))] = np.array([1, 0, 0], f)
    elif mode == 2:
        with np.errstate(divide="ignore", invalid="ignore", over="ignore"):
            t = (m - f(min_mass)) / (f(max_mass) - f(min_mass))
            one_t = f(1) - t
            # (1 - t) * (0, 0, 1) + t * (1, 0, 0), product then sum per component
            col[:, 0] = one_t * f(0) + t * f(1)
            col[:, 1] = one_t * f(0) + t * f(0)
            col[:, 2] = one_t * f(1) + t * f(0)
            special = np.array([np.float64(np.inf), 214.0 / 255.0, 160.0 / 255.0]).astype(f)
        col[m == 0] = special
    return pos.copy(), col


def animation_advance(state: dict, dt, walls=None) -> dict:
    """updateAnimation's decisions (main.cu:1210-1262) restated on a dict of
    AnimationState's fields, in float32 arithmetic operation by operation.
    Returns the frame's move: translation, rotation (degrees), center and
    whether animateParticles runs."""
    F = np.float32
    dt = F(dt)
    move = {"translation": np.zeros(3, F), "rotation": F(0), "center": np.zeros(3, F), "apply": 0}
    if not state["is_animating"]:
        return move
    state["animation_time"] = F(F(state["animation_time"]) + dt)
    tr = np.zeros(3, F)
    rot = F(0)
    if state["animation_time"] <= F(2.5) and not state["translation_complete"]:
        d = np.asarray(state["translation_direction"], F)
        tr = np.array([F(F(d[k] * F(state["translation_speed"])) * dt) for k in range(3)], F)
    elif not state["translation_complete"]:
        state["translation_complete"] = 1
        state["animation_time"] = F(0)
        cen = np.zeros(3, F)
        count = 0
        for i in range(state["start_index"], state["start_index"] + state["num_particles"]):
            cen = np.array([F(cen[k] + F(walls[i][k])) for k in range(3)], F)
            count += 1
        if count > 0:
            state["rotation_center"] = np.array([F(cen[k] / F(count)) for k in range(3)], F)
    if state["translation_complete"] and F(state["rotation_angle"]) < F(45.0):
        delta = F(-F(state["rotation_speed"]) * dt)
        state["rotation_angle"] = F(F(state["rotation_angle"]) + abs(delta))
        rot = delta
        if state["rotation_angle"] >= F(45.0):
            state["is_animating"] = 0
    move.update(translation=tr, rotation=rot, center=np.asarray(state["rotation_center"], F).copy(),
                apply=1 if state["is_animating"] else 0)
    return move
