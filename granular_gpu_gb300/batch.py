"""Batched scenes: many independent scenes stepped by one system.

The batched-scenes configuration: 64 box-drop / pile scenes with particle
counts drawn log-uniform in [10,000, 500,000] (seeded), radius 0.005,
friction U[0.3, 0.7], stepped together.  law="coulomb" (the default) runs
the configured mode with the friction as each scene's static Coulomb
coefficient (kinetic 0.8 of it) and its box faces as analytic walls in the
scene's own coordinates; law="cap" runs the reference's contact law with the
friction as each scene's tangential cap.  Scene k sits in the slab
k*W <= x < (k+1)*W (W = its 1 m box plus a gap of two cells), so one grid,
one sort and one launch of each kernel serve all scenes and no contact
crosses scenes (gg_set_scenes); a frame of substeps is captured once into a
CUDA graph and replayed with one launch (gg_graph_capture).
"""
import math

import numpy as np

from . import GranularSystem, abi, workloads, _check, lib
import ctypes as C

R = 0.005
BOX = 1.0
DT = 1.0 / 240.0


def _scene(rng, n: int, r: float = R):
    """One scene in a BOX^3 box: a jittered block of about n particles
    (spacing 2r) released between 0.02 and 0.3 above the floor."""
    a = max(2, int(round(n ** (1.0 / 3.0))))
    b = max(2, int(round(n / (a * a))))
    counts = (a, b, a)
    span = [(c - 1) * 2 * r for c in counts]
    drop = float(rng.uniform(0.02, 0.3))
    origin = (BOX / 2 - span[0] / 2, 0.005 * BOX + 0.01 * (r / 0.01) + r + drop, BOX / 2 - span[2] / 2)
    p = workloads.lattice(counts, 2 * r, origin, 0.05 * r, int(rng.integers(1 << 30)))
    return p


def batched_scenes(n_scenes: int = 64, seed: int = 0, lo: int = 10_000, hi: int = 500_000, r: float = R,
                   law: str = "coulomb"):
    """(desc, info) of a batch: desc for GranularSystem(...); info holds the
    slab width, per-scene friction and particle ranges."""
    rng = np.random.default_rng(seed)
    L = np.float32(workloads.CELL_PER_RADIUS * r)
    counts = np.exp(rng.uniform(math.log(lo), math.log(hi), n_scenes)).astype(np.int64)
    fric = rng.uniform(0.3, 0.7, n_scenes).astype(np.float32)
    walls1, cs1 = workloads.box_walls((BOX, BOX, BOX), L)
    W = float(np.float32(BOX + 2 * float(L)))
    parts, walls, sizes = [], [], []
    for k in range(n_scenes):
        p = _scene(rng, int(counts[k]), r)
        off = np.array([k * W, 0.0, 0.0], np.float32)
        parts.append(p + off)
        walls.append(walls1 + off)
        sizes.append(p.shape[0])
    particles = np.concatenate(parts).astype(np.float32)
    boundary = np.concatenate(walls).astype(np.float32)
    space = (n_scenes * W, BOX, BOX)
    cell_size = (int(math.ceil(space[0] / float(L))), cs1[1], cs1[2])
    params = workloads.scaled_params(r, iters=5)
    params.upsample_enabled = 0
    params.merge_enabled = 0
    if law == "coulomb":
        workloads.configure(params, 0.5, 0.4, workloads.box_planes((BOX, BOX, BOX)))
    elif law != "cap":
        raise ValueError(law)
    desc = workloads._desc(particles, boundary, None, space, L, cell_size, DT, (0.0, -9.81, 0.0),
                           workloads.density_for_radius(r), 0, params, skip=True)
    info = {"n_scenes": n_scenes, "width": W, "friction_cap": fric, "sizes": np.array(sizes),
            "walls_per_scene": walls1.shape[0], "law": law}
    return desc, info


def scene_desc(desc, info, k: int):
    """The desc of scene k alone (its own 1 m box at the origin)."""
    sizes = info["sizes"]
    a = int(sizes[:k].sum())
    b = a + int(sizes[k])
    nw = info["walls_per_scene"]
    off = np.array([k * info["width"], 0.0, 0.0], np.float32)
    p = (desc["particles"][a:b] - off).astype(np.float32)
    w = (desc["boundary"][k * nw:(k + 1) * nw] - off).astype(np.float32)
    L = np.float32(desc["cell_length"])
    _, cs = workloads.box_walls((BOX, BOX, BOX), L)
    params = abi.gg_params()
    C.memmove(C.byref(params), C.byref(desc["params"]), C.sizeof(params))
    params.friction_cap = float(info["friction_cap"][k])
    if info.get("law") == "coulomb":
        params.mu_static = float(info["friction_cap"][k])
        params.mu_kinetic = float(np.float32(0.8) * info["friction_cap"][k])
    return workloads._desc(p, w, None, (BOX, BOX, BOX), L, cs, desc["dt"], desc["gravity"], desc["density"], 0,
                           params, skip=True)


class Batch:
    """A batch of scenes in one system, with per-scene friction and FP64
    per-scene diagnostics."""

    def __init__(self, desc, info, device: int = 0):
        self.info = info
        self.system = GranularSystem(**workloads.system_kwargs(desc), device=device)
        fc = np.ascontiguousarray(info["friction_cap"], np.float32)
        _check(lib().gg_set_scenes(self.system._h, info["n_scenes"], info["width"],
                                   fc.ctypes.data_as(C.POINTER(C.c_float))))
        if info.get("law") == "coulomb":
            mus = fc
            muk = np.ascontiguousarray(np.float32(0.8) * fc, np.float32)
            self._mu = (mus, muk)
            _check(lib().gg_set_scene_coulomb(self.system._h, info["n_scenes"],
                                              mus.ctypes.data_as(C.POINTER(C.c_float)),
                                              muk.ctypes.data_as(C.POINTER(C.c_float))))

    def scene_stats(self) -> np.ndarray:
        """n_scenes x 9: count, mass, momentum xyz, kinetic energy, centre of mass xyz (FP64)."""
        n = self.info["n_scenes"]
        out = np.zeros((n, 9), np.float64)
        _check(lib().gg_scene_stats(self.system._h, out.ctypes.data_as(C.POINTER(C.c_double)), n))
        return out

    def autotune(self, substeps: int = 4) -> dict:
        """gg_autotune: the fastest launch shapes for this batch."""
        return self.system.autotune(substeps)

    def capture(self, substeps: int):
        _check(lib().gg_graph_capture(self.system._h, substeps))

    def launch(self):
        _check(lib().gg_graph_launch(self.system._h))

    def close(self):
        self.system.close()


def measure(n_scenes: int = 64, frames: int = 10, substeps: int = 4, seed: int = 0, device: int = 0,
            sequential: bool = True, law: str = "coulomb") -> dict:
    """Aggregate particle-substeps/s of the batch replayed as a CUDA graph
    (one launch per frame of `substeps` substeps), of the same batch stepped
    substep by substep, and of the scenes as separate systems stepped one
    after another on one stream (per-scene launches).  Every arm starts from
    the same initial state, runs one untimed frame, then `frames` timed
    frames; device time with CUDA events on the stream it runs on."""
    import torch
    desc, info = batched_scenes(n_scenes, seed=seed, law=law)
    n_total = int(desc["n_particles"])
    units = n_total * substeps * frames
    out = {"scenes": n_scenes, "particles": n_total, "frames": frames, "substeps_per_frame": substeps,
           "contact_law": law,
           "boundary_particles": int(desc["n_boundary"]), "cells": int(np.prod(desc["cell_size"]))}

    def timed(stream, fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        fn()  # warm-up frame
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(frames):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    b = Batch(desc, info, device=device)
    ms = timed(torch.cuda.ExternalStream(b.system.stream, device=device), lambda: b.system.step(substeps))
    out["batched_launches"] = units / (ms / 1e3)
    b.close()
    b = Batch(desc, info, device=device)
    out["autotune"] = b.autotune(substeps)
    b.capture(substeps)
    ms = timed(torch.cuda.ExternalStream(b.system.stream, device=device), b.launch)
    out["batched_graph"] = units / (ms / 1e3)
    stats = b.scene_stats()
    out["scene_diagnostics_fp64"] = {"max_abs_momentum": float(np.abs(stats[:, 2:5]).max()),
                                     "total_kinetic_energy": float(stats[:, 5].sum()),
                                     "particles_per_scene_min_max": [int(stats[:, 0].min()), int(stats[:, 0].max())]}
    b.close()
    if sequential:
        stream = torch.cuda.Stream(device=device)
        systems = [GranularSystem(**workloads.system_kwargs(scene_desc(desc, info, k)), device=device,
                                  stream=stream.cuda_stream) for k in range(n_scenes)]

        def frame():
            for x in systems:
                x.step(substeps)

        ms = timed(stream, frame)
        for x in systems:
            x.close()
        out["sequential"] = units / (ms / 1e3)
        out["speedup_vs_sequential"] = out["batched_graph"] / out["sequential"]
    return out
