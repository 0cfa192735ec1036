"""granular_gpu_gb300 — GB300-native granular substep path behind a C ABI.

Python mirror of the reference's GranularSystem surface
(src/GranularSystem.hpp:8-56, src/Particles.hpp, src/GranularParticles.hpp),
built only on libgg.so (include/gg.h).  There is no CPU fallback: every
call runs the CUDA library and raises if it is missing.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import (FIELD_ADAPTIVE_LAST_STEP, FIELD_CELL_KEY, FIELD_CELL_START,  # noqa: F401
                  FIELD_CONTACTS, FIELD_FEATURES, FIELD_IS_ANIMATED, FIELD_WARM_TARGET, FIELD_MASS, FIELD_MASS_UNITS, FIELD_MERGE,
                  FIELD_MERGE_COUNT, FIELD_MERGE_VELOCITY, FIELD_NUM_CONSTRAINTS, FIELD_PERM,
                  FIELD_POS, FIELD_REMOVE, FIELD_SURFACE, FIELD_SURFACE_DISTANCE, FIELD_VEL,
                  SET_BOUNDARY, SET_GRANULAR, SET_UPSAMPLED, default_params)

__all__ = ["GranularSystem", "GranularError", "Grid", "Mlp", "scene_build", "default_params", "lib"]

_LIB = None


def lib() -> C.CDLL:
    """The loaded libgg.so (raises abi.NativeLibraryMissing when unbuilt)."""
    global _LIB
    if _LIB is None:
        _LIB = abi.load_library()
    return _LIB


class GranularError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


def _check(rc: int):
    if rc != abi.GG_OK:
        msg = lib().gg_last_error()
        raise GranularError(rc, msg.decode() if msg else "")


def _f32(a, comp=3):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).reshape(-1, comp))


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32)) if a is not None else None


class ParticleSet:
    """get_*_ptr() readers of one particle set (Particles.hpp:18-20,
    GranularParticles.hpp:19-26), copying to host arrays."""

    def __init__(self, system: "GranularSystem", which: int):
        self._s = system
        self._set = which

    def size(self) -> int:
        return self._s._size(self._set)

    def get_pos(self):
        return self._s.read(FIELD_POS, self._set)

    def get_vel(self):
        return self._s.read(FIELD_VEL, self._set)

    def get_mass(self):
        return self._s.read(FIELD_MASS, self._set)

    def get_surface(self):
        return self._s.read(FIELD_SURFACE, self._set)

    def get_surface_distance(self):
        return self._s.read(FIELD_SURFACE_DISTANCE, self._set)

    def get_adaptive_last_step(self):
        return self._s.read(FIELD_ADAPTIVE_LAST_STEP, self._set)

    def get_particle_2_cell(self):
        return self._s.read(FIELD_CELL_KEY, self._set)

    def get_is_animated(self):
        return self._s.read(FIELD_IS_ANIMATED, self._set)


class Solver:
    """GranularSystem::get_solver() (GranularSystem.hpp:56)."""

    def __init__(self, system: "GranularSystem"):
        self._s = system

    def save_particle_stats(self, filename: str):
        _check(lib().gg_save_particle_stats(self._s._h, filename.encode()))

    def trigger_explosion(self, explosion_force: float):
        _check(lib().gg_trigger_explosion(self._s._h, float(explosion_force)))

    def get_buffer_merge_count(self):
        return self._s.read(FIELD_MERGE_COUNT)

    def get_buffer_merge(self):
        return self._s.read(FIELD_MERGE)

    def get_buffer_remove(self):
        return self._s.read(FIELD_REMOVE)


class GranularSystem:
    """GranularSystem(particles, boundary, upsampled, space_size, cell_length,
    dt, g, cell_size, density, upsampled_radius, is_move_boundary,
    is_adaptive) — GranularSystem.hpp:8-14.  Construction runs one step, as
    the reference's constructor does (GranularSystem.cu:62)."""

    def __init__(self, particles, boundary_particles, upsampled_particles, space_size, cell_length,
                 dt, g, cell_size, density, upsampled_radius=0.005, is_move_boundary=False,
                 is_adaptive=1, *, masses=None, boundary_animated=None, params=None, device=0,
                 max_particles=0, skip_initial_step=False, stream=None):
        self._h = None
        l = lib()
        p = _f32(particles)
        b = _f32(boundary_particles) if boundary_particles is not None and len(boundary_particles) else None
        u = _f32(upsampled_particles) if upsampled_particles is not None and len(upsampled_particles) else None
        m = np.ascontiguousarray(masses, dtype=np.float32) if masses is not None else None
        a = np.ascontiguousarray(boundary_animated, dtype=np.int32) if boundary_animated is not None else None
        d = abi.gg_desc()
        d.particles, d.n_particles = _fptr(p), p.shape[0]
        d.masses = _fptr(m)
        d.boundary, d.n_boundary = _fptr(b), 0 if b is None else b.shape[0]
        d.boundary_animated = _iptr(a)
        d.upsampled, d.n_upsampled = _fptr(u), 0 if u is None else u.shape[0]
        for i in range(3):
            d.space_size[i] = float(space_size[i])
            d.gravity[i] = float(g[i])
            d.cell_size[i] = int(cell_size[i])
        d.cell_length, d.dt, d.density = float(cell_length), float(dt), float(density)
        d.upsampled_radius = float(upsampled_radius)
        d.is_move_boundary, d.is_adaptive = int(bool(is_move_boundary)), int(is_adaptive)
        d.skip_initial_step, d.device = int(bool(skip_initial_step)), int(device)
        d.max_particles = int(max_particles)
        d.stream = stream
        d.params = params if params is not None else default_params()
        h = C.c_void_p()
        _check(l.gg_create(C.byref(d), C.byref(h)))
        self._h = h
        self.device = int(device)
        self.cell_size = tuple(int(x) for x in cell_size)

    @classmethod
    def from_scene(cls, json_path: str, params=None, device=0, base_dir=None, max_particles=0,
                   skip_initial_step=False, stream=None) -> "GranularSystem":
        """loadSceneConfig + init_granular_system + constructor
        (main.cu:123-167, 746-1173)."""
        self = cls.__new__(cls)
        self._h = None
        ov = abi.gg_overrides()
        if params is not None:
            ov.has_params, ov.params = 1, params
        ov.device, ov.max_particles, ov.stream = int(device), int(max_particles), stream
        ov.skip_initial_step = int(bool(skip_initial_step))
        ov.base_dir = base_dir.encode() if base_dir else None
        h = C.c_void_p()
        _check(lib().gg_create_from_scene(json_path.encode(), C.byref(ov), C.byref(h)))
        self._h = h
        self.device = int(device)
        cs = (C.c_int32 * 3)()
        _check(lib().gg_grid_dims(h, cs, None))
        self.cell_size = tuple(cs)
        return self

    # -- GranularSystem::step and sizes ---------------------------------
    def step(self, n_substeps: int = 1) -> int:
        _check(lib().gg_step(self._h, int(n_substeps)))
        return 1

    def synchronize(self):
        _check(lib().gg_synchronize(self._h))

    def _size(self, which):
        n = C.c_int64()
        _check(lib().gg_size(self._h, which, C.byref(n)))
        return n.value

    def size(self) -> int:
        return self._size(SET_GRANULAR)

    def upsampled_size(self) -> int:
        return self._size(SET_UPSAMPLED)

    def boundary_size(self) -> int:
        return self._size(SET_BOUNDARY)

    def total_size(self) -> int:
        return self.size() + self.boundary_size() + self.upsampled_size()

    def get_particles(self) -> ParticleSet:
        return ParticleSet(self, SET_GRANULAR)

    def get_boundaries(self) -> ParticleSet:
        return ParticleSet(self, SET_BOUNDARY)

    def get_upsampled(self) -> ParticleSet:
        return ParticleSet(self, SET_UPSAMPLED)

    def get_solver(self) -> Solver:
        return Solver(self)

    # -- field access -----------------------------------------------------
    def read(self, field: int, which: int = SET_GRANULAR, out=None):
        dt, comp = abi.FIELD_LAYOUT[field]
        n = C.c_int64()
        _check(lib().gg_read(self._h, which, field, None, 0, C.byref(n)))
        cnt = n.value
        if out is None:
            out = np.empty((max(cnt, 1), comp), dtype=dt)
        _check(lib().gg_read(self._h, which, field, out.ctypes.data_as(C.c_void_p), out.shape[0], C.byref(n)))
        out = out[:cnt]
        return out[:, 0] if comp == 1 else out

    def write(self, field: int, data, which: int = SET_GRANULAR):
        a = _f32(data)
        _check(lib().gg_write(self._h, which, field, a.ctypes.data_as(C.c_void_p), a.shape[0]))

    def device_ptr(self, field: int, which: int = SET_GRANULAR):
        p, n, st = C.c_void_p(), C.c_int64(), C.c_int32()
        _check(lib().gg_device_ptr(self._h, which, field, C.byref(p), C.byref(n), C.byref(st)))
        return p.value, n.value, st.value

    @property
    def params(self) -> "abi.gg_params":
        """A copy of the parameters in use (gg_get_params)."""
        p = abi.gg_params()
        _check(lib().gg_get_params(self._h, C.byref(p)))
        return p

    @params.setter
    def params(self, p):
        _check(lib().gg_set_params(self._h, C.byref(p)))

    # -- learned warm start -------------------------------------------------
    def color_buffer(self, mode: int = 2, which: int = SET_GRANULAR, min_mass: float = 1.0,
                     max_mass: float = 4.0, out=None):
        """gg_color_buffer: (dots, colors), each an (n, 3) float32 array, as the
        reference's generate_dots writes them into its vertex buffers.  `out`
        may give two CUDA tensors of 3 * n floats to fill on the device
        instead (returned as they are, after the system's stream has run)."""
        import torch
        n = self._size(which)
        if out is None:
            dots = torch.empty(max(3 * n, 1), dtype=torch.float32, device=f"cuda:{self.device}")
            cols = torch.empty_like(dots)
        else:
            dots, cols = out
        _check(lib().gg_color_buffer(self._h, which, mode, min_mass, max_mass,
                                     C.c_void_p(dots.data_ptr()), C.c_void_p(cols.data_ptr())))
        self.synchronize()
        if out is not None:
            return dots, cols
        return (dots[: 3 * n].view(n, 3).cpu().numpy(), cols[: 3 * n].view(n, 3).cpu().numpy())

    def autotune(self, substeps: int = 2) -> dict:
        """gg_autotune: the fastest launch shapes and default-sweep variant
        for this system's current state (the state is left as it was)."""
        t = abi.gg_tuning()
        _check(lib().gg_autotune(self._h, substeps, C.byref(t)))
        return {k: getattr(t, k) for k, _ in abi.gg_tuning._fields_ if k != "pad_"}

    def tuning(self) -> dict:
        """gg_get_tuning: the launch shapes and default-sweep variant in use."""
        t = abi.gg_tuning()
        _check(lib().gg_get_tuning(self._h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in abi.gg_tuning._fields_ if k != "pad_"}

    def set_tuning(self, **changes):
        """gg_set_tuning: change some launch shapes (for example the ones an
        earlier autotune chose); results do not depend on them."""
        t = abi.gg_tuning()
        _check(lib().gg_get_tuning(self._h, C.byref(t)))
        for k, v in changes.items():
            if k not in dict(abi.gg_tuning._fields_):
                raise KeyError(k)
            setattr(t, k, v)
        _check(lib().gg_set_tuning(self._h, C.byref(t)))

    def set_warm_start(self, mlp=None):
        """gg_set_warm_start: attach a network (gg_params.warm_start = 1) or,
        with None, only allocate the buffers of the recording mode (2)."""
        _check(lib().gg_set_warm_start(self._h, mlp.handle if mlp is not None else None))
        self._mlp = mlp

    # -- diagnostics, snapshots, timing ----------------------------------
    def stats(self) -> dict:
        s = abi.gg_stats_t()
        _check(lib().gg_stats(self._h, C.byref(s)))
        out = {k: getattr(s, k) for k, _ in abi.gg_stats_t._fields_}
        for k in ("momentum", "center_of_mass"):
            out[k] = tuple(out[k])
        return out

    def write_vtk(self, path: str, which: int = SET_UPSAMPLED, swap_yz: bool = True):
        """ASCII VTK point cloud (the reference's writers, main.cu:190-254)."""
        _check(lib().gg_write_vtk(self._h, which, path.encode(), int(bool(swap_yz))))

    def write_vtk_centered(self, path: str, which: int = SET_UPSAMPLED):
        """saveUpsampledPositionsToVTK (main.cu:588-664)."""
        _check(lib().gg_write_vtk_centered(self._h, which, path.encode()))

    def write_vtk_by_mass(self, base: str, frame_id: int):
        """saveParticlesByMass (main.cu:256-368)."""
        _check(lib().gg_write_vtk_by_mass(self._h, base.encode(), int(frame_id)))

    def write_vtk_animated_boundary(self, path: str, centred: bool = True):
        """saveBoundaryParticlesToVTK / saveFunnelBoundaryParticlesToVTK
        (main.cu:434-527 / 370-432)."""
        _check(lib().gg_write_vtk_animated_boundary(self._h, path.encode(), int(bool(centred))))

    def write_vtk_points_centered(self, points, path: str):
        """saveAdditionalBoundaryParticlesToVTK (main.cu:529-586)."""
        a = _f32(points)
        _check(lib().gg_write_vtk_points_centered(self._h, a.ctypes.data_as(C.c_void_p), a.shape[0], path.encode()))

    def write_csv(self, path: str, which: int = SET_UPSAMPLED):
        """saveUpsampledPositionsToCSV (main.cu:673-694)."""
        _check(lib().gg_write_csv(self._h, which, path.encode()))

    def write_frame_times(self, path: str):
        """saveFrameTimes (main.cu:665-671)."""
        _check(lib().gg_write_frame_times(self._h, path.encode()))

    def save(self, path: str):
        _check(lib().gg_save(self._h, path.encode()))

    def load(self, path: str):
        _check(lib().gg_load(self._h, path.encode()))

    def set_frame_timing(self, enabled: bool = True):
        _check(lib().gg_set_frame_timing(self._h, int(bool(enabled))))

    def get_frame_times(self):
        n = C.c_int64()
        _check(lib().gg_frame_times(self._h, None, 0, C.byref(n)))
        out = np.zeros(max(n.value, 1), np.float32)
        _check(lib().gg_frame_times(self._h, _fptr(out), out.shape[0], C.byref(n)))
        return out[:n.value]

    def graph_capture(self, substeps: int):
        """Records `substeps` substeps (an even number) into a CUDA graph
        (gg_graph_capture); only for substeps without host round trips (no
        merge/split, no residual mode)."""
        _check(lib().gg_graph_capture(self._h, int(substeps)))

    def graph_launch(self):
        """Replays the captured substeps with one launch (gg_graph_launch)."""
        _check(lib().gg_graph_launch(self._h))

    def update_animation(self, state: "abi.gg_animation", dt: float):
        """updateAnimation (main.cu:1210-1277): advances `state` by one frame
        of dt and moves the animated walls (before the frame's substeps)."""
        _check(lib().gg_update_animation(self._h, C.byref(state), C.c_float(dt)))

    def animate_walls(self, move: "abi.gg_animation_move"):
        """animateParticles (main.cu:1175-1208) with the given move."""
        _check(lib().gg_animate_walls(self._h, C.byref(move)))

    def profile_begin(self):
        _check(lib().gg_profile_begin(self._h))

    def profile_end(self) -> dict:
        p = abi.gg_profile_t()
        _check(lib().gg_profile_end(self._h, C.byref(p)))
        out = {}
        for k in range(p.n_classes):
            name = bytes(p.names[k]).split(b"\0")[0].decode()
            out[name] = {"launches": p.launches[k], "ms": p.ms[k], "units": p.units[k]}
        out["_kernel_launches"] = p.kernel_launches
        out["_nlist_rebuilds"] = p.nlist_rebuilds
        return out

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        _check(lib().gg_stream(self._h, C.byref(s)))
        return s.value or 0

    def close(self):
        if getattr(self, "_h", None):
            lib().gg_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def scene_build(json_path: str, base_dir: str = None) -> dict:
    """The particle sets and constructor arguments of a scene file, built on
    the host (init_granular_system, main.cu:746-1173)."""
    l = lib()
    np_, nb, nu = C.c_int64(), C.c_int64(), C.c_int64()
    bd = base_dir.encode() if base_dir else None
    _check(l.gg_scene_build(json_path.encode(), bd, None, C.byref(np_), None, None, C.byref(nb), None,
                            C.byref(nu), None))
    p = np.zeros((max(np_.value, 1), 3), np.float32)
    b = np.zeros((max(nb.value, 1), 3), np.float32)
    a = np.zeros(max(nb.value, 1), np.int32)
    u = np.zeros((max(nu.value, 1), 3), np.float32)
    d = abi.gg_desc()
    _check(l.gg_scene_build(json_path.encode(), bd, _fptr(p), C.byref(np_), _fptr(b), _iptr(a), C.byref(nb),
                            _fptr(u), C.byref(nu), C.byref(d)))
    return {
        "particles": p[:np_.value], "boundary": b[:nb.value], "boundary_animated": a[:nb.value],
        "upsampled": u[:nu.value], "space_size": tuple(d.space_size), "cell_length": d.cell_length,
        "dt": d.dt, "gravity": tuple(d.gravity), "cell_size": tuple(d.cell_size), "density": d.density,
        "upsampled_radius": d.upsampled_radius, "is_move_boundary": d.is_move_boundary,
        "is_adaptive": d.is_adaptive, "params": d.params,
    }


def default_animation() -> "abi.gg_animation":
    """AnimationState's initialisers (main.cu:100-111), not animating."""
    a = abi.gg_animation()
    _check(lib().gg_default_animation(C.byref(a)))
    return a


def scene_animation(json_path: str, base_dir: str = None) -> "abi.gg_animation":
    """The animation state a scene's construction leaves (the excavator's
    and the funnel's obj_file walls)."""
    a = abi.gg_animation()
    bd = base_dir.encode() if base_dir else None
    _check(lib().gg_scene_animation(json_path.encode(), bd, C.byref(a)))
    return a


def animation_advance(state: "abi.gg_animation", dt: float, walls=None) -> "abi.gg_animation_move":
    """updateAnimation's host part: advances `state` and returns the frame's
    move; `walls` (float[3] per wall particle) is read when the translation
    phase ends."""
    m = abi.gg_animation_move()
    if walls is None:
        w, n = None, 0
    else:
        w = _f32(walls)
        n = w.shape[0]
    _check(lib().gg_animation_advance(C.byref(state), C.c_float(dt), None if w is None else _fptr(w), n,
                                      C.byref(m)))
    return m


class Grid:
    """Stand-alone grid build (keys, stable sort, cell ranges) on the GPU."""

    def __init__(self, capacity: int, cell_size, cell_length: float, device: int = 0):
        self._h = None
        cs = (C.c_int32 * 3)(*[int(x) for x in cell_size])
        h = C.c_void_p()
        _check(lib().gg_grid_create(int(device), int(capacity), cs, float(cell_length), C.byref(h)))
        self._h = h
        self.cell_size = tuple(int(x) for x in cell_size)

    def build(self, pos):
        p = _f32(pos)
        n = p.shape[0]
        ncell = self.cell_size[0] * self.cell_size[1] * self.cell_size[2]
        keys = np.zeros(max(n, 1), np.int32)
        sk = np.zeros(max(n, 1), np.int32)
        perm = np.zeros(max(n, 1), np.int32)
        cs = np.zeros(ncell + 1, np.int32)
        _check(lib().gg_grid_build(self._h, _fptr(p), n, _iptr(keys), _iptr(sk), _iptr(perm), _iptr(cs)))
        return keys[:n], sk[:n], perm[:n], cs

    def close(self):
        if getattr(self, "_h", None):
            lib().gg_grid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _dptr(t):
    """Device address of a torch CUDA tensor (or an int address)."""
    if t is None:
        return None
    if isinstance(t, int):
        return C.c_void_p(t)
    return C.c_void_p(t.data_ptr())


class Mlp:
    """The warm-start network (gg_mlp_*): 48 -> 64 -> 64 -> 3, ReLU, BF16
    tensor-core kernels with FP32 accumulation.  Feature and target arrays
    are device memory (torch CUDA tensors or raw addresses): features n x 48
    bf16, targets n x 3 float32."""

    N_FEATURES, N_HIDDEN, N_OUT = 48, 64, 3

    def __init__(self, device: int = 0, seed: int = 1):
        self.device = device
        h = C.c_void_p()
        _check(lib().gg_mlp_create(device, seed, C.byref(h)))
        self._h = h

    @staticmethod
    def num_params() -> int:
        return int(lib().gg_mlp_num_params())

    @property
    def handle(self):
        return self._h

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.num_params(), np.float32)
        _check(lib().gg_mlp_get_params(self._h, _fptr(out), out.size))
        return out

    def set_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float32)
        _check(lib().gg_mlp_set_params(self._h, _fptr(p), p.size))

    def forward(self, features, out, n: int, stream=None):
        _check(lib().gg_mlp_forward(self._h, _dptr(features), n, _dptr(out), stream))

    def gradient(self, features, targets, n: int, stream=None):
        g = np.zeros(self.num_params(), np.float32)
        loss = C.c_float()
        _check(lib().gg_mlp_gradient(self._h, _dptr(features), _dptr(targets), n, _fptr(g), C.byref(loss),
                                     stream))
        return g, float(loss.value)

    def train_step(self, features, targets, n: int, lr: float, weight_decay: float = 0.0, stream=None) -> float:
        loss = C.c_float()
        _check(lib().gg_mlp_train_step(self._h, _dptr(features), _dptr(targets), n, lr, weight_decay,
                                       C.byref(loss), stream))
        return float(loss.value)

    def close(self):
        if getattr(self, "_h", None):
            lib().gg_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
