"""The reference's own CUDA kernels, driven from Python (TEST INFRASTRUCTURE ONLY).

Only tests/ and bench.py's reference arm (`--impl reference`, which times
the reference's own kernels) may import this module.  It loads the cubins that
`oracle/ref_cuda_build.py` compiled from the reference's `src/Solver.cu` and
`src/GranularSystem.cu` (unmodified) through the CUDA driver API, launches the
reference's `__global__` kernels with the reference's launch shapes
(`(num - 1) / block_size + 1` blocks of `block_size` = 256, `Global.hpp:5`)
on the legacy default stream, and restates the host orchestration around
them:

* the grid build of `GranularSystem::neighbor_search_granular`
  (`src/GranularSystem.cu:65-173`): `mapParticles2Cells_CUDA`, a stable sort
  by key (the reference's `thrust::sort_by_key` on int keys is a stable radix
  sort), the gathers of velocity and mass, `countingInCell_CUDA` and an
  exclusive scan over C+1 counts;
* the boundary and upsampled grids (`src/GranularSystem.cu:174-395`);
* `Solver::step` (`src/Solver.cu:82-109`): the thrust functors
  `add_external_force`, `predict_position_functor`, `mass_scaling_functor`,
  `change_position_functor` and `final_velocity_functor` (`:125-270`,
  `:403-414`) restated as elementwise torch operations, each with the
  functor's own operation order, around the reference's `compute_delta_pos`
  (`:361-401`) in the reference's 3 stabilisation + `max_iter` = 5 sweeps
  (`Solver::project`, `:416-513`);
* `Solver::upsampled_update` (`:1371-1387`) -> `update_upsampled_cuda`;
* `GranularSystem::set_surface_particles` and `find_distance_to_surface`
  (`src/GranularSystem.cu:613-699`) -> `find_cover_vector`, `find_surface`,
  `compute_distance_to_surface`;
* `Solver::adaptive_sampling` (`src/Solver.cu:856-1242`) -> `merge_mark_gpu`,
  `merge_count_gpu`, `split_gpu`, `extract_split_particles_kernel`, with the
  compaction and append of `DArray` / `GranularParticles` restated;
* `generate_dots` (`src/VBO.hpp:96-106`) -> `generate_dots_CUDA`, the colouring
  of the vertex buffers.

The torch restatements of the functors round as the reference's device code
does when it is built with `-fmad=false` (the `_nofma` cubins).  With the
reference's own flags (FMA contraction on) the kernels in the cubin contract
multiply-adds, and the functors here do not: results then agree to rounding.
"""
import ctypes as C
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
BLOCK = 256  # block_size, Global.hpp:5

# argument kinds of each reference kernel, in its parameter order
_SIGS = {
    "mapParticles2Cells_CUDA": "p p f i3 i",
    "countingInCell_CUDA": "p p i",
    "compute_delta_pos": "p p p p p i p p i3 f i p",
    "update_upsampled_cuda": "p p p p p i p p p i3 f",
    "find_cover_vector": "p p p i p i3 f f",
    "find_surface": "p p p p i p i3 f f",
    "compute_distance_to_surface": "i p p p i3 f p",
    "generate_dots_CUDA": "p p p i p p f f i p",
    "merge_mark_gpu": "i p p p p p p p p p p f i3 f p",
    "merge_count_gpu": "i p p p p p p i p",
    "split_gpu": "i p p p p p p p p p f i3 p p f f p",
    "extract_split_particles_kernel": "p p p p i",
}
_UNIT_OF = {
    "mapParticles2Cells_CUDA": "solver", "countingInCell_CUDA": "solver",
    "compute_delta_pos": "solver", "update_upsampled_cuda": "solver",
    "find_cover_vector": "gsystem", "find_surface": "gsystem",
    "compute_distance_to_surface": "gsystem",
    "generate_dots_CUDA": "vbo",
    "merge_mark_gpu": "solver", "merge_count_gpu": "solver", "split_gpu": "solver",
    "extract_split_particles_kernel": "solver",
}
# struct SplitParticle (Solver.cu:701-706): float3 pos, float3 vel, float mass,
# bool valid -> 29 bytes, padded to 32 (4-byte alignment)
SPLIT_PARTICLE_BYTES = 32


class _Int3(C.Structure):
    _fields_ = [("x", C.c_int32), ("y", C.c_int32), ("z", C.c_int32)]


def available() -> bool:
    return os.path.exists(os.path.join(REF_DIR, "entries.json"))


class _Driver:
    """The few CUDA driver calls the harness needs, through ctypes."""

    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")
        for name, args in {
            "cuInit": [C.c_uint],
            "cuCtxGetCurrent": [C.POINTER(C.c_void_p)],
            "cuModuleLoad": [C.POINTER(C.c_void_p), C.c_char_p],
            "cuModuleUnload": [C.c_void_p],
            "cuModuleGetFunction": [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p],
            "cuLaunchKernel": [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                               C.c_uint, C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)],
            "cuCtxSynchronize": [],
            "cuGetErrorString": [C.c_int, C.POINTER(C.c_char_p)],
        }.items():
            fn = getattr(self.cu, name)
            fn.argtypes = args
            fn.restype = C.c_int

    def check(self, rc: int, what: str):
        if rc != 0:
            s = C.c_char_p()
            self.cu.cuGetErrorString(rc, C.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} ({(s.value or b'?').decode()})")


class RefKernels:
    """The reference's kernels from one flavour of the cubins: `fma=True`
    loads the build with the reference's own flags, `fma=False` the build
    with -fmad=false."""

    def __init__(self, fma: bool = False):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.torch = torch
        self.d = _Driver()
        self.d.check(self.d.cu.cuInit(0), "cuInit")
        ctx = C.c_void_p()
        self.d.check(self.d.cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        with open(os.path.join(REF_DIR, "entries.json")) as f:
            entries = json.load(f)
        suffix = "" if fma else "_nofma"
        self.mods = {}
        self.fns = {}
        for unit in ("solver", "gsystem", "vbo"):
            name = f"{unit}{suffix}.cubin"
            mod = C.c_void_p()
            self.d.check(self.d.cu.cuModuleLoad(C.byref(mod), os.path.join(REF_DIR, name).encode()),
                         f"cuModuleLoad {name}")
            self.mods[unit] = (mod, entries[name])
        for k, unit in _UNIT_OF.items():
            mod, ent = self.mods[unit]
            fn = C.c_void_p()
            self.d.check(self.d.cu.cuModuleGetFunction(C.byref(fn), mod, ent[k].encode()),
                         f"cuModuleGetFunction {k}")
            self.fns[k] = fn

    def launch(self, name: str, num: int, *args):
        """Launches kernel `name` over `num` threads with the reference's
        launch shape; tensor arguments are passed as device pointers."""
        kinds = _SIGS[name].split()
        assert len(kinds) == len(args), (name, len(kinds), len(args))
        if num <= 0:
            return
        vals = []
        for kind, a in zip(kinds, args):
            if kind == "p":
                vals.append(C.c_uint64(a.data_ptr() if a is not None else 0))
            elif kind == "i":
                vals.append(C.c_int32(int(a)))
            elif kind == "f":
                vals.append(C.c_float(float(a)))
            elif kind == "i3":
                vals.append(_Int3(int(a[0]), int(a[1]), int(a[2])))
            else:
                raise ValueError(kind)
        params = (C.c_void_p * len(vals))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
        grid = (num - 1) // BLOCK + 1
        self.d.check(self.d.cu.cuLaunchKernel(self.fns[name], grid, 1, 1, BLOCK, 1, 1, 0, None, params, None),
                     f"launch {name}")

    def synchronize(self):
        self.d.check(self.d.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    def close(self):
        for mod, _ in self.mods.values():
            self.d.cu.cuModuleUnload(mod)
        self.mods = {}


def _f32(x) -> float:
    """x rounded to float32, as a Python float (exactly representable)."""
    return float(np.float32(x))


class RefSystem:
    """The reference's per-step path on the reference's own kernels.

    State is float3 AoS in device tensors, as the reference keeps it.
    `step()` follows `GranularSystem::step` (`src/GranularSystem.cu:397-453`)
    for a non-moving boundary: granular and upsampled grid builds (which
    permute velocity, mass and the solver's merge, merge-count and remove
    buffers, `:90-145`), `Solver::step`, `Solver::upsampled_update` and, when
    `adaptive`, the surface and distance kernels and
    `Solver::adaptive_sampling` (`src/Solver.cu:856-1242`): `merge_mark_gpu`
    on every call but the first (`t_merge_iter`, `:36,910-922`; kept per
    system here, per process there), `merge_count_gpu`, `split_gpu` with its
    atomic append into a zero-filled SplitParticle buffer, the stable
    compaction of mass, adaptive_last_step, position, velocity, merge count,
    merge and remove by `remove == 1` (`DArray::compact`,
    `src/DArray.hpp:62-113`; merge_velocity is not compacted), and the append
    of the split children through `extract_split_particles_kernel` with
    adaptive_last_step 1 and zero solver buffers
    (`src/GranularParticles.hpp:48-88`).  `max_mass` is the constructor's
    `_max_mass(4)` (`src/GranularSystem.cu:49`), an argument of the merge and
    split kernels.
    """

    def __init__(self, k: RefKernels, pos, vel, mass, bpos, upos=None, uvel=None, *, cell_size,
                 cell_length, dt, gravity, density, max_iter=5, stab_iters=3, adaptive=False,
                 max_mass=4.0, blend_factor=40):
        torch = k.torch
        self.k, self.t = k, torch
        dev = "cuda"
        f = lambda a: torch.as_tensor(np.ascontiguousarray(a, np.float32), device=dev).contiguous()
        self.pos = f(pos).reshape(-1, 3)
        self.vel = f(vel).reshape(-1, 3)
        self.mass = f(mass).reshape(-1)
        self.bpos = f(bpos).reshape(-1, 3)
        self.upos = f(upos).reshape(-1, 3) if upos is not None else None
        self.uvel = f(uvel).reshape(-1, 3) if uvel is not None else None
        self.cs = tuple(int(c) for c in cell_size)
        self.C = self.cs[0] * self.cs[1] * self.cs[2]
        self.L = _f32(cell_length)
        self.dt = _f32(dt)
        self.G = [_f32(g) for g in gravity]
        self.density = _f32(density)
        self.max_iter = max_iter
        self.stab_iters = stab_iters
        self.adaptive = adaptive
        self.max_mass = _f32(max_mass)
        self.blend_factor = int(blend_factor)
        n = self.pos.shape[0]
        self.als = torch.zeros(n, dtype=torch.int32, device=dev)
        # the solver's buffers (Solver.hpp:108-113), zero-filled like every DArray
        self.remove = torch.zeros(n, dtype=torch.int32, device=dev)
        self.merge = torch.zeros(n, dtype=torch.float32, device=dev)
        self.merge_count = torch.zeros(n, dtype=torch.int32, device=dev)
        self.merge_vel = torch.zeros((max(n, 1), 3), dtype=torch.float32, device=dev)
        self.merge_lock = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
        self.num_surface = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
        self.t_merge_iter = 0
        self.stats = []  # (removed, split, count before) per adaptive step, Solver.cu:1234-1235
        self.last_n = None
        self.surface = None
        self.surface_distance = None
        # the constructor's boundary grid (GranularSystem.cu:56)
        self.bpos, _, self.cs_b = self.grid(self.bpos)

    def set_adaptive_last_step(self, flags):
        """adaptive_last_step is not permuted by the grid sort
        (`src/GranularSystem.cu:90-145` gathers every other field), so it
        stays with its array slot."""
        self.als = self.t.as_tensor(np.ascontiguousarray(flags, np.int32), device="cuda").contiguous()

    def set_solver_buffers(self, remove, merge, merge_count, merge_velocity):
        """Solver::_buffer_remove, _merge, _merge_count, _merge_velocity."""
        t = self.t
        self.remove = t.as_tensor(np.ascontiguousarray(remove, np.int32), device="cuda").contiguous()
        self.merge = t.as_tensor(np.ascontiguousarray(merge, np.float32), device="cuda").contiguous()
        self.merge_count = t.as_tensor(np.ascontiguousarray(merge_count, np.int32), device="cuda").contiguous()
        mv = np.ascontiguousarray(merge_velocity, np.float32).reshape(-1, 3)
        if mv.shape[0] < self.merge_vel.shape[0]:
            mv = np.concatenate([mv, np.zeros((self.merge_vel.shape[0] - mv.shape[0], 3), np.float32)])
        self.merge_vel = t.as_tensor(mv, device="cuda").contiguous()

    def size(self) -> int:
        return int(self.pos.shape[0])

    # -- neighbour search (GranularSystem.cu:65-173, 174-280, 282-395)
    def keys(self, pos):
        torch = self.t
        n = pos.shape[0]
        keys = torch.empty(max(n, 1), dtype=torch.int32, device="cuda")
        self.k.launch("mapParticles2Cells_CUDA", n, keys, pos, self.L, self.cs, n)
        return keys[:n]

    def cell_start(self, sorted_keys):
        torch = self.t
        n = sorted_keys.shape[0]
        counts = torch.zeros(self.C + 1, dtype=torch.int32, device="cuda")
        self.k.launch("countingInCell_CUDA", n, counts, sorted_keys.contiguous(), n)
        cs = torch.zeros(self.C + 1, dtype=torch.int64, device="cuda")
        cs[1:] = torch.cumsum(counts[:-1].to(torch.int64), 0)
        return cs.to(torch.int32)

    def grid(self, pos):
        """Keys, stable sort by key, cell start; returns (sorted positions,
        permutation, cell start)."""
        torch = self.t
        keys = self.keys(pos)
        skeys, perm = torch.sort(keys, stable=True)
        return pos[perm].contiguous(), perm, self.cell_start(skeys)

    def neighbor_search(self):
        self.pos, perm, self.cs_g = self.grid(self.pos)
        self.vel = self.vel[perm].contiguous()
        self.mass = self.mass[perm].contiguous()
        self.merge = self.merge[perm].contiguous()
        self.merge_count = self.merge_count[perm].contiguous()
        self.remove = self.remove[perm].contiguous()
        self.perm = perm
        if self.upos is not None and self.upos.shape[0]:
            keys = self.keys(self.upos)
            _, up = self.t.sort(keys, stable=True)
            self.upos = self.upos[up].contiguous()
            self.uvel = self.uvel[up].contiguous()
            self.cs_u = self.cell_start(keys[up])

    # -- Solver::step (Solver.cu:82-109)
    def solver_step(self):
        torch = self.t
        n = self.pos.shape[0]
        dv = torch.tensor([_f32(np.float32(self.dt) * np.float32(g)) for g in self.G],
                          dtype=torch.float32, device="cuda")
        self.vel = self.vel + dv                                         # add_external_force
        self.pos_t = self.pos + self.dt * self.vel                       # predict_position_functor
        self.scaled_mass = self.mass * torch.exp(-self.pos[:, 1])        # mass_scaling_functor
        delta = torch.zeros((max(n, 1), 3), dtype=torch.float32, device="cuda")
        ncon = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
        dens_int = int(self.density)  # compute_delta_pos takes `const int density`

        def sweep():
            delta.zero_()
            ncon.zero_()
            self.k.launch("compute_delta_pos", n, delta, ncon, self.pos_t, self.bpos, self.mass, n,
                          self.cs_g, self.cs_b, self.cs, self.L, dens_int, self.scaled_mass)
            d = delta[:n] / torch.clamp(ncon[:n], min=1).to(torch.float32)[:, None]
            return d

        for _ in range(self.stab_iters):                                 # Solver.cu:428-467 (3)
            d = sweep()
            self.pos = self.pos + d
            self.pos_t = self.pos_t + d
        for _ in range(self.max_iter):                                   # Solver.cu:469-512
            d = sweep()
            self.pos_t = self.pos_t + d
        self.last_n = ncon[:n].clone()
        # final_velocity_functor (Solver.cu:193-248)
        dt_inv = _f32(np.float32(1.0) / np.float32(self.dt))
        v = dt_inv * (self.pos_t - self.pos)
        speed = torch.sqrt(v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2])
        span = _f32(np.float32(10.0) - np.float32(1.0))
        t = torch.clamp((speed - 1.0) / span, 0.0, 1.0)
        damping = 0.99 + (_f32(np.float32(0.99) - np.float32(0.99))) * t
        damping = damping.to(torch.float32)
        one_minus = (1.0 - damping)
        fac = damping + one_minus * torch.exp((-speed) * _f32(0.1))
        damped = v * fac[:, None]
        damped = torch.where((self.als == 1)[:, None], damped * _f32(0.98), damped)
        v = torch.where((speed > 1.0)[:, None], damped, v)
        v = torch.where((speed < _f32(0.01))[:, None], torch.zeros_like(v), v)
        self.vel = v.contiguous()
        self.pos = self.pos_t.clone()                                    # final_update memcpy
        self.als.zero_()

    def upsampled_update(self):
        if self.upos is None or not self.upos.shape[0]:
            return
        nu = self.upos.shape[0]
        self.k.launch("update_upsampled_cuda", nu, self.upos, self.pos, self.bpos, self.vel, self.uvel, nu,
                      self.cs_u, self.cs_g, self.cs_b, self.cs, self.L)

    def surface_pass(self):
        torch = self.t
        n = self.pos.shape[0]
        cover = torch.zeros((max(n, 1), 3), dtype=torch.float32, device="cuda")
        surf = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
        dist = torch.zeros(max(n, 1), dtype=torch.float32, device="cuda")
        self.k.launch("find_cover_vector", n, cover, self.pos, self.mass, n, self.cs_g, self.cs, self.L,
                      self.density)
        self.k.launch("find_surface", n, surf, cover, self.pos, self.mass, n, self.cs_g, self.cs, self.L,
                      self.density)
        self.k.launch("compute_distance_to_surface", n, n, self.pos, surf, self.cs_g, self.cs, self.L, dist)
        self.surface = surf[:n]
        self.surface_distance = dist[:n]

    # -- Solver::adaptive_sampling (Solver.cu:856-1242)
    def adaptive_sampling(self):
        torch = self.t
        n = self.size()
        if n == 0:
            return
        if self.merge_vel.shape[0] < n:  # the reference's buffer keeps its first length
            extra = torch.zeros((n - self.merge_vel.shape[0], 3), dtype=torch.float32, device="cuda")
            self.merge_vel = torch.cat([self.merge_vel, extra]).contiguous()
            self.merge_lock = torch.zeros(n, dtype=torch.int32, device="cuda")
            self.num_surface = torch.zeros(n, dtype=torch.int32, device="cuda")
        if self.t_merge_iter == 1:
            self.k.launch("merge_mark_gpu", n, n, self.pos, self.mass, self.vel, self.surface,
                          self.surface_distance, self.num_surface, self.remove, self.merge, self.merge_vel,
                          self.cs_g, self.max_mass, self.cs, self.L, self.merge_lock)
            self.t_merge_iter = 0
        self.t_merge_iter += 1
        self.k.launch("merge_count_gpu", n, n, self.merge, self.mass, self.vel, self.merge_count, self.remove,
                      self.merge_vel, self.blend_factor, self.als)
        splits = torch.zeros(n * SPLIT_PARTICLE_BYTES // 4, dtype=torch.int32, device="cuda")
        split_count = torch.zeros(1, dtype=torch.int32, device="cuda")
        self.k.launch("split_gpu", n, n, self.pos, self.mass, self.vel, self.bpos, self.surface, self.remove,
                      self.merge, self.cs_g, self.cs_b, self.max_mass, self.cs, splits, split_count, self.density,
                      self.L, self.als)
        keep = self.remove != 1
        removed = int(n - int(keep.sum().item()))
        if removed:
            self.mass = self.mass[keep].contiguous()
            self.als = self.als[keep].contiguous()
            self.pos = self.pos[keep].contiguous()
            self.vel = self.vel[keep].contiguous()
            self.merge_count = self.merge_count[keep].contiguous()
            self.merge = self.merge[keep].contiguous()
            self.remove = self.remove[keep].contiguous()
        ns = int(split_count.item())
        if ns > 0:
            m_new = torch.zeros(ns, dtype=torch.float32, device="cuda")
            p_new = torch.zeros((ns, 3), dtype=torch.float32, device="cuda")
            v_new = torch.zeros((ns, 3), dtype=torch.float32, device="cuda")
            self.k.launch("extract_split_particles_kernel", ns, splits, m_new, p_new, v_new, ns)
            self.mass = torch.cat([self.mass, m_new]).contiguous()
            self.als = torch.cat([self.als, torch.ones(ns, dtype=torch.int32, device="cuda")]).contiguous()
            self.pos = torch.cat([self.pos, p_new]).contiguous()
            self.vel = torch.cat([self.vel, v_new]).contiguous()
            zi = torch.zeros(ns, dtype=torch.int32, device="cuda")
            self.remove = torch.cat([self.remove, zi]).contiguous()
            self.merge_count = torch.cat([self.merge_count, zi]).contiguous()
            self.merge = torch.cat([self.merge, torch.zeros(ns, dtype=torch.float32, device="cuda")]).contiguous()
        self.stats.append((removed, ns, n))

    def step(self, sync: bool = True):
        self.neighbor_search()
        self.solver_step()
        self.upsampled_update()
        if self.adaptive:
            self.surface_pass()
            self.adaptive_sampling()
        if sync:
            self.k.synchronize()

    def read(self, name: str):
        return getattr(self, name).detach().cpu().numpy()
