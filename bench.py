"""Benchmark: particle-substeps/s of the column-collapse workload on GB300.

A "step" is one substep of the reference's GranularSystem::step (grid
build, 3 stabilisation + 4 Jacobi sweeps, finalize, upsampling of 4 render
points per particle, surface detection and merge/split up to mass 8) over
8,388,608 particles resident in HBM, with the reference's length constants
as compiled into its kernels.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]

The headline window is substeps 40 .. 40+K of the collapse, where the first
merges complete (a merge blends over 40 substeps) and the particle count
starts to fall; the K substeps right after the W warm-up substeps are
reported beside it as `early_window`.

N > 1 runs N independent replicas (one per rank, launched by torchrun); the
path has no exchange step.  `--impl reference` times the reference's own
CUDA kernels (its Solver.cu and GranularSystem.cu compiled unmodified for
sm_103a with its own device flags, driven by oracle/ref_cuda.py, which
restates its thrust calls in torch) on the same scene, windows and host
copies; this library is not loaded in that arm.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-substeps/s"
WORKLOAD = "column collapse 128x256x256 (8,388,608 particles, r=0.002, 2x1x1 box, dt=1/120 x 4 substeps, " \
           "3+4 sweeps, merge/split to mass 8, 4 render points/particle, the reference's length constants " \
           "as compiled into its kernels)"
WINDOW_START = 40  # the headline window starts at this substep (the constructor's is substep 1)
SAMPLE_COUNTS = (64, 64, 64)
SAMPLE_NOTE = "64x64x64 sub-lattice (262,144 particles) of the same column scene (same box, grid, walls, " \
              "parameters), one oracle substep per step"
# Algorithmic (compulsory) bytes per unit of each kernel class, with FP32
# float3 state and neighbour re-reads assumed to hit in cache: the roofline
# is reported for whichever class takes the most time in the timed region.
ALGO_BYTES = {
    "sweep": (40, "particle", "read x* and contact radius 16 B, inverse mass 4 B and cell key 4 B; write the "
                              "correction and its counts 16 B"),
    "upsample": (48, "render point", "read render-point position and velocity 24 B, write them 24 B"),
    "surface": (20, "particle", "read position and radius 16 B, write the surface flag 4 B"),
    "apply": (56, "particle", "read correction 16 B and x* 12 B, write x* 12 B (stabilisation: x 12 B more), "
                              "count 4 B"),
    "merge": (24, "particle", "read position and radius 16 B, surface distance 4 B, write the mark 4 B"),
}


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.out.flush()
        rows = []
        with open(self.out.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.out.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def stream_kernels(prof: dict, desc: dict, peak: float) -> dict:
    """The HBM-bound grid classes, timed live like the dominant kernel:
    algorithmic bytes per unit (P radix passes of 8 bits over keys up to C:
    16 B per scatter pass, 4 B per histogram pass after the first, whose
    digits the hash kernel counts), achieved GB/s and the fraction of the
    measured copy bandwidth."""
    passes = max(1, -(-int(np.prod(desc["cell_size"])).bit_length() // 8))
    sort_b = 16 * passes + 4 * (passes - 1)
    basis = {
        "hash": (24, "particle", "read position 16 B, write key and index 8 B"),
        "sort": (sort_b, "particle", f"{passes} scatter passes of key and index, {passes - 1} histogram passes"),
        "reorder": (124, "particle", "gather 9 per-particle fields by the permutation (read and write)"),
        "up_grid": (24 + sort_b + 68, "render point",
                    "hash 24 B, sort, then gather index 4 B and position and velocity 32 B in, 32 B out"),
    }
    out = {}
    for k, (b, unit, note) in basis.items():
        v = prof.get(k)
        if not v or not v["launches"] or v["ms"] <= 0:
            continue
        gbs = b * v["units"] / (v["ms"] / 1e3) / 1e9
        out[k] = {"bytes_per_unit": b, "unit_of_work": unit, "bytes_basis": note,
                  "achieved_gbs": round(gbs, 1), "frac": round(gbs / peak, 3)}
    return out


def ncu_traffic(cls: str):
    """DRAM bytes per launch of a kernel class from one ncu capture
    (dram__bytes_read.sum + dram__bytes_write.sum) and the units that launch
    processed, from the committed summary; None when it has no entry."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d.get(cls)
    except (OSError, ValueError):
        return None


def reduce_over_ranks(ms: float, units: float, device: str = "cuda"):
    """Replicas: the job takes as long as its slowest rank (max of the
    timed milliseconds) and processes the units of all ranks (sum)."""
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    import torch.distributed as tdist
    if tdist.is_available() and tdist.is_initialized() and tdist.get_world_size() > 1:
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        tdist.all_reduce(u, op=tdist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def cpu_sample(steps: int, warmup: int, fp64: bool = True):
    """Times the oracle (CPU restatement) on the bounded sample."""
    from granular_gpu_gb300 import workloads
    from oracle import oracle as orc
    desc = workloads.column_collapse(counts=SAMPLE_COUNTS, constants="reference")
    o = orc.OracleSystem(desc, fp64=fp64)
    o.step(warmup)
    units = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        units += o.size()
        o.step(1)
    dt = time.perf_counter() - t0
    threads = orc.threads()
    o.close()
    return units / dt, threads, dt


def fp64_error(device: int) -> dict:
    """The library (FP32, CUDA's own math functions) against the serial FP64
    restatement after one substep (the constructor's) from the same state of
    the bounded sample: max |x - x_fp64| in units of r, its 99.9th
    percentile and the particles beyond 1e-3 r, and max |v - v_fp64|.  The
    FP32 restatement against the FP64 one is reported beside it: with the
    reference's wall reach (0.02 = 2.5 cells at r = 0.002) a particle near a
    cell face sees different wall particles when a rounding moves it across
    the face (the stencil covers one cell each way), so a few particles
    differ by a good part of r in any FP32 build.  (After a second grid
    build the two sort particles near cell faces differently, so particles
    compare index by index after one substep.)"""
    import granular_gpu_gb300 as gg
    from granular_gpu_gb300 import abi, workloads
    from oracle import oracle as orc
    desc = workloads.column_collapse(counts=SAMPLE_COUNTS, constants="reference")
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=device)
    o = orc.OracleSystem(desc, fp64=True)
    o32 = orc.OracleSystem(desc, fp64=False)
    r = 0.002

    def err(pos, vel):
        d = np.abs(pos.astype(np.float64) - o.read(abi.FIELD_POS).astype(np.float64)).max(1) / r
        dv = np.abs(vel.astype(np.float64) - o.read(abi.FIELD_VEL).astype(np.float64)).max()
        return {"pos_max_abs_r": float(d.max()), "pos_p999_abs_r": float(np.quantile(d, 0.999)),
                "particles_over_1e-3_r": int((d > 1e-3).sum()), "vel_max_abs": float(dv)}

    if s.size() != o.size() or o32.size() != o.size():
        out = {"unavailable": f"particle counts differ ({s.size()}, {o32.size()} vs {o.size()})"}
    else:
        out = err(s.read(gg.FIELD_POS), s.read(gg.FIELD_VEL))
        out.update({"substeps": 1, "particles": int(o.size()),
                    "sample": "64x64x64 sub-lattice of the column scene, FP32 CUDA math against the FP64 build",
                    "fp32_oracle_vs_fp64": err(o32.read(abi.FIELD_POS), o32.read(abi.FIELD_VEL))})
    s.close()
    o.close()
    o32.close()
    return out


def _line_base(args, world, value, ms, dtype, config):
    return {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": config}


def _config(desc, counts, world, impl_note):
    return {"workload": WORKLOAD if counts == (128, 256, 256) else f"column collapse {counts}",
            "particles": desc["n_particles"], "upsampled": desc["n_upsampled"], "boundary": desc["n_boundary"],
            "cells": int(np.prod(desc["cell_size"])),
            "window": f"substeps {WINDOW_START}..{WINDOW_START}+K of the collapse (the first merges complete at "
                      f"substep 41); the K substeps after the W warm-up substeps are `early_window`",
            "l2": "inputs larger than L2 (about 1.9 GB of particle state per step)",
            "parallelism": f"replicas x{world}", "implementation": impl_note}


def run_reference(args):
    """The reference's own CUDA kernels on the headline workload: the same
    scene, windows and host copies as the library's arm.  This library is
    never loaded here."""
    rank, world, local = _dist()
    if rank != 0:
        return 0
    import torch
    from oracle import ref_cuda
    if not ref_cuda.available():
        print(json.dumps({"impl": "reference", "unavailable": "the reference's kernels were not compiled "
                          "(oracle/_ref/ is empty: no reference checkout where build() ran)"}), flush=True)
        return 0
    from granular_gpu_gb300 import workloads
    torch.cuda.set_device(local)
    counts = tuple(int(c) for c in args.counts.split(","))
    desc = workloads.column_collapse(counts=counts, seed=42, constants="reference")
    P = desc["params"]
    n0, nu = desc["n_particles"], desc["n_upsampled"]
    k = ref_cuda.RefKernels(fma=True)  # the reference's own device flags
    r = ref_cuda.RefSystem(k, desc["particles"], np.zeros((n0, 3), np.float32), np.ones(n0, np.float32),
                           desc["boundary"], desc["upsampled"], np.zeros((nu, 3), np.float32),
                           cell_size=desc["cell_size"], cell_length=desc["cell_length"], dt=desc["dt"],
                           gravity=desc["gravity"], density=desc["density"], max_iter=P.iters,
                           stab_iters=P.stab_iters, adaptive=True, max_mass=P.max_mass)
    r.step()  # the constructor's step (GranularSystem.cu:62)
    done = 1
    for _ in range(args.warmup):
        r.step()
        done += 1

    def window(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        units = 0
        e0.record()
        for _ in range(steps):
            units += r.size()
            r.step()  # ends with a device synchronisation, as GranularSystem::step does
        e1.record()
        torch.cuda.synchronize()
        return units, e0.elapsed_time(e1)

    eu, ems = window(args.steps)
    done += args.steps
    early = {"value": eu / (ems / 1e3), "ms_per_step": ems / args.steps,
             "substeps": f"{2 + args.warmup}..{1 + args.warmup + args.steps}", "particles_now": r.size()}
    while done < WINDOW_START - 1:
        r.step()
        done += 1
    sampler = ClockSampler(local)
    sampler.start()
    n_before = r.size()
    units, ms = window(args.steps)
    clocks = sampler.stop()
    value = units / (ms / 1e3)
    removed = sum(x[0] for x in r.stats)
    split = sum(x[1] for x in r.stats)
    # end to end: the caller's cudaMemcpy of positions and velocities into the
    # reference's device arrays before each step and of positions,
    # velocities and render points out of them after it (main.cu:206-209)
    # pinned host buffers sized once (each step uses the leading rows)
    cap = 2 * n0
    hp_all = torch.empty((cap, 3), dtype=torch.float32, pin_memory=True)
    hv_all = torch.empty((cap, 3), dtype=torch.float32, pin_memory=True)
    hu = torch.empty((r.upos.shape[0], 3), dtype=torch.float32, pin_memory=True)
    m = r.size()
    hp_all[:m].copy_(r.pos)
    hv_all[:m].copy_(r.vel)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_units = h2d = d2h = 0
    for _ in range(args.steps):
        r.pos.copy_(hp_all[:m], non_blocking=True)
        r.vel.copy_(hv_all[:m], non_blocking=True)
        h2d += 2 * m * 12
        e2e_units += m
        r.step()
        m = r.size()
        hp_all[:m].copy_(r.pos, non_blocking=True)
        hv_all[:m].copy_(r.vel, non_blocking=True)
        hu.copy_(r.upos, non_blocking=True)
        torch.cuda.synchronize()
        d2h += 2 * m * 12 + hu.shape[0] * 12
    e2e_s = time.perf_counter() - t0
    line = _line_base(args, 1, value, ms, "f32", _config(
        desc, counts, 1, "the reference's Solver.cu and GranularSystem.cu kernels compiled unmodified for sm_103a "
                         "with its own device flags (oracle/_ref/solver.cubin, gsystem.cubin), launched with its "
                         "launch shapes by oracle/ref_cuda.py, which restates its thrust calls and host "
                         "orchestration in torch (no per-step allocation, which favours the reference); "
                         "max_iter 4 and max_mass 8 as the configuration states (literals 5 and 4 there)"))
    line["impl"] = "reference"
    line["early_window"] = early
    line["window"] = {"particles_start": n_before, "particles_now": r.size(), "merged_total": removed,
                      "split_total": split}
    line["e2e"] = {"value": e2e_units / e2e_s, "unit": METRIC, "h2d_bytes_per_step": h2d // max(args.steps, 1),
                   "d2h_bytes_per_step": d2h // max(args.steps, 1)}
    line["gpu_launches"] = None  # the reference's kernels, not this library's
    line["clocks"] = clocks
    k.close()
    if not args.no_cpu:
        # the reference has no CPU implementation of the path: its FP64
        # restatement on the host cores, on the bounded sample
        cv, threads, _ = cpu_sample(steps=args.cpu_steps, warmup=1)
        line["cpu_baseline"] = {"value": cv, "unit": METRIC, "cores": threads, "kind": "port",
                                "sample": SAMPLE_NOTE + f", {args.cpu_steps} timed substeps, FP64 build"}
    print(json.dumps(line), flush=True)
    return 0


def pile_rate(device: int, steps: int) -> dict:
    import torch
    import granular_gpu_gb300 as gg
    from granular_gpu_gb300 import workloads
    desc = workloads.adaptive_pile()
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=device)
    s.step(100)
    s.synchronize()
    tune = s.autotune(2)
    st = torch.cuda.ExternalStream(s.stream, device=device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    units = 0
    e0.record(st)
    for _ in range(steps):
        units += s.size()
        s.step(1)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    stats = s.stats()
    s.close()
    return {"metric": METRIC, "value": units / (ms / 1e3), "ms_per_step": ms / steps, "steps": steps,
            "particles_start": desc["n_particles"], "particles_now": stats["n_particles"],
            "render_points": desc["n_upsampled"], "merged_total": stats["merged_total"],
            "split_total": stats["split_total"],
            "mass_units_conserved": stats["total_mass_units"] == desc["n_particles"] * (1 << 20),
            "autotune": {k: tune[k] for k in ("sweep_variant", "keep_threads", "build_blocks_per_sm", "trials",
                                              "ms_default", "ms_tuned")},
            "workload": "64^3 block (r = 0.005, spacing 2r) dropped 0.02 onto the floor of a 2x1x1 box with a "
                        "30-degree ramp of wall particles, dt = 1/240, 3+5 sweeps, merge/split to mass 8, "
                        "4 render points per particle, the reference's length constants; autotuned (gg_autotune) "
                        "and timed after 100 substeps"}


def box_drop_rate(device: int) -> dict:
    """The box-drop configuration as stated (configured mode): 32^3
    particles, r = 0.01, dt = 1/60 in 4 substeps, 3 Jacobi sweeps, Coulomb
    friction 0.5 / 0.4, restitution 0, box faces as analytic walls; all 300
    frames timed (device time, CUDA events), stepped substep by substep and,
    from the same start, each frame's 4 substeps replayed as one CUDA graph
    (the scene has no merge/split, so a frame needs no host round trip)."""
    import torch
    import granular_gpu_gb300 as gg
    from granular_gpu_gb300 import workloads
    frames = 300
    out = {}
    for mode in ("stepped", "graph"):
        desc = workloads.box_drop(n_side=32, substeps=4, iters=3, configured=True)
        s = gg.GranularSystem(**workloads.system_kwargs(desc), device=device)
        if mode == "graph":
            s.graph_capture(4)
        st = torch.cuda.ExternalStream(s.stream, device=device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(frames):
            if mode == "graph":
                s.graph_launch()
            else:
                s.step(4)
        e1.record(st)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        stats = s.stats()
        p = s.read(gg.FIELD_POS)
        out[mode] = {"ms": ms, "nonfinite": stats["nonfinite"], "pos": p}
        s.close()
    n = desc["n_particles"]
    g, t = out["graph"], out["stepped"]
    return {"metric": METRIC, "value": n * 4 * frames / (g["ms"] / 1e3), "ms_per_frame": g["ms"] / frames,
            "stepped_value": n * 4 * frames / (t["ms"] / 1e3), "stepped_ms_per_frame": t["ms"] / frames,
            "graph_equals_stepping": bool(np.array_equal(g["pos"], t["pos"])),
            "frames": frames, "substeps": 4 * frames, "particles": n, "nonfinite": g["nonfinite"],
            "inside_box": bool(np.all(g["pos"] >= 0.005) and np.all(g["pos"] <= 0.995)),
            "workload": "32^3 box drop (r = 0.01, lattice 2r, jitter 0.05r, block centred 0.5 above the floor), "
                        "dt = 1/60 in 4 substeps, 3 Jacobi sweeps, Coulomb friction 0.5 / 0.4, restitution 0, "
                        "box faces as analytic walls (configured mode), 300 frames from rest, each frame one "
                        "CUDA-graph launch"}


def scaled_rate(device: int, counts, warmup: int, steps: int) -> dict:
    """The same column with every length constant scaled by r / 0.01 (a
    configuration of this library the reference's compiled-in constants
    cannot run), timed right after the warm-up."""
    import torch
    import granular_gpu_gb300 as gg
    from granular_gpu_gb300 import workloads
    desc = workloads.column_collapse(counts=counts, seed=42, constants="scaled")
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=device)
    s.step(warmup)
    s.synchronize()
    st = torch.cuda.ExternalStream(s.stream, device=device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    units = 0
    e0.record(st)
    for _ in range(steps):
        units += s.size()
        s.step(1)
    e1.record(st)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    s.close()
    return {"metric": METRIC, "value": units / (ms / 1e3), "ms_per_step": ms / steps, "steps": steps,
            "substeps": f"{2 + warmup}..{1 + warmup + steps}",
            "workload": "the headline column with wall reach, merge radius, upsampling support and floor scaled "
                        "by r / 0.01 and render points advected with the substep's dt"}


def run_mine(args):
    import torch
    import granular_gpu_gb300 as gg
    from granular_gpu_gb300 import workloads

    rank, world, local = _dist()
    dist_on = world > 1
    if dist_on:
        import torch.distributed as tdist
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    counts = tuple(int(c) for c in args.counts.split(","))
    desc = workloads.column_collapse(counts=counts, seed=42 + rank, constants="reference")
    if args.math_mode:
        desc["params"].math_mode = args.math_mode
    if args.nlist_skin is not None:
        desc["params"].nlist_skin = args.nlist_skin * 0.002
    n0 = desc["n_particles"]
    sysg = gg.GranularSystem(**workloads.system_kwargs(desc), device=local)  # substep 1
    stream = torch.cuda.ExternalStream(sysg.stream, device=local)
    done = 1
    for _ in range(args.warmup):
        sysg.step(1)
        done += 1
    sysg.synchronize()

    def barrier():
        if dist_on:
            tdist.barrier()

    def window(steps):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        units = 0
        ev0.record(stream)
        for _ in range(steps):
            units += sysg.size()
            sysg.step(1)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return units, ev0.elapsed_time(ev1)

    # ---- early window: the K substeps after the warm-up
    eu, ems = window(args.steps)
    done += args.steps
    ems_max, eu_total = reduce_over_ranks(ems, eu)
    early = {"value": eu_total / (ems_max / 1e3), "ms_per_step": ems_max / args.steps,
             "substeps": f"{2 + args.warmup}..{1 + args.warmup + args.steps}", "particles_now": sysg.size()}
    while done < WINDOW_START - 1:
        sysg.step(1)
        done += 1
    sysg.synchronize()
    st0 = sysg.stats()

    # ---- headline window, device-resident
    sampler = ClockSampler(local)
    sampler.start()
    sysg.profile_begin()
    units, ms = window(args.steps)
    prof = sysg.profile_end()
    launches = prof.pop("_kernel_launches")
    list_builds = prof.pop("_nlist_rebuilds")
    clocks = sampler.stop()
    st1 = sysg.stats()
    ms_max, total_units = reduce_over_ranks(ms, units)
    value = total_units / (ms_max / 1000.0)

    # ---- end to end through the C ABI with pinned host buffers
    if args.no_e2e:
        args.steps_e2e = 0
    else:
        args.steps_e2e = args.steps
    # pinned host buffers sized once for the system's capacity (the particle
    # count changes every substep once merges complete; each step uses the
    # leading rows)
    cap = max(2 * n0, sysg.size())
    nu = sysg.upsampled_size()
    hp_all = torch.empty((cap, 3), dtype=torch.float32, pin_memory=True).numpy()
    hv_all = torch.empty((cap, 3), dtype=torch.float32, pin_memory=True).numpy()
    hu = torch.empty((nu, 3), dtype=torch.float32, pin_memory=True).numpy()
    m = sysg.size()
    sysg.read(gg.FIELD_POS, out=hp_all[:m])
    sysg.read(gg.FIELD_VEL, out=hv_all[:m])
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_units = 0
    h2d = d2h = 0
    step_evs = []
    for _ in range(args.steps_e2e):
        # this step's inputs from the host, the step, its results back
        sysg.write(gg.FIELD_POS, hp_all[:m])
        sysg.write(gg.FIELD_VEL, hv_all[:m])
        h2d += 2 * 12 * m
        e2e_units += m
        ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ea.record(stream)
        sysg.step(1)
        eb.record(stream)
        step_evs.append((ea, eb))
        m = sysg.size()
        sysg.read(gg.FIELD_POS, out=hp_all[:m])
        sysg.read(gg.FIELD_VEL, out=hv_all[:m])
        sysg.read(gg.FIELD_POS, gg.SET_UPSAMPLED, out=hu)
        d2h += 2 * 12 * m + hu.nbytes
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_s_max, e2e_total = reduce_over_ranks(e2e_s, e2e_units)
    e2e_value = e2e_total / e2e_s_max if args.steps_e2e else None
    # the same substeps' device time alone (CUDA events around each step on
    # the library's stream): what the copies and the host add is the rest
    e2e_step_ms = sum(a.elapsed_time(b) for a, b in step_evs)

    # ---- roofline of the dominant kernel class
    known = {k: v for k, v in prof.items() if k in ALGO_BYTES and v["launches"]}
    dom = max(known.items(), key=lambda kv: kv[1]["ms"])[0]
    kp = prof[dom]
    per_unit, unit_name, byte_note = ALGO_BYTES[dom]
    peak, peak_kind = measured_peak()
    avg_ms = kp["ms"] / max(kp["launches"], 1)
    units_per_launch = kp["units"] / max(kp["launches"], 1)
    algo_bytes = per_unit * units_per_launch
    achieved = algo_bytes / (avg_ms / 1000.0) / 1e9
    tr = ncu_traffic(dom)
    traffic = None
    if tr and tr.get("units"):
        # traffic grows with the units processed: scale the captured launch
        traffic = float(tr["dram_bytes"]) * units_per_launch / float(tr["units"])
    total_ms = sum(v["ms"] for v in prof.values())
    shares = {k: round(v["ms"] / total_ms, 4) for k, v in prof.items() if v["launches"]}

    line = _line_base(args, world, value, ms_max, "f32", _config(
        desc, counts, world, "this library (granular_gpu_gb300/_build/libgg.so), integer mass ledger"))
    line.update({
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_unit": per_unit, "unit_of_work": unit_name,
                     "bytes_basis": byte_note, "units_per_launch": units_per_launch,
                     "avg_launch_ms": avg_ms, "shares": shares,
                     # the same ncu capture's issue figures: the stencil kernels are
                     # bound by instruction issue, not by HBM
                     "issue_active_pct": (tr or {}).get("issue_active_pct"),
                     "sm_throughput_pct": (tr or {}).get("sm_throughput_pct"),
                     "list_builds_per_particle_sweep": list_builds / max(prof["sweep"]["units"], 1),
                     "stream_kernels": stream_kernels(prof, desc, peak)},
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d // max(args.steps, 1),
                "d2h_bytes_per_step": d2h // max(args.steps, 1),
                "ms_per_step": e2e_s_max * 1e3 / max(args.steps_e2e, 1),
                "device_ms_per_step": e2e_step_ms / max(args.steps_e2e, 1),
                "device_only_value": (e2e_units / (e2e_step_ms / 1e3)) if args.steps_e2e and e2e_step_ms > 0
                else None,
                "substeps": f"{WINDOW_START + args.steps}..{WINDOW_START + 2 * args.steps - 1}"},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "early_window": early,
        "window": {"particles_start": st0["n_particles"], "particles_now": st1["n_particles"],
                   "merged_total": st1["merged_total"], "split_total": st1["split_total"],
                   "merged_in_window": st1["merged_total"] - st0["merged_total"],
                   "mass_units_conserved": st1["total_mass_units"] == n0 * (1 << 20)},
    })
    if rank == 0 and world == 1 and not args.no_scaled:
        line["column_scaled_constants"] = scaled_rate(local, counts, args.warmup, args.steps)
    if rank == 0 and world == 1 and not args.no_pile:
        # the adaptive-pile configuration: 262,144 particles of r = 0.005 on the
        # floor of a box with a 30-degree ramp, merge/split to mass 8 on the
        # integer ledger, 4 render points per particle; timed after 100
        # substeps (merges under way)
        line["adaptive_pile"] = pile_rate(local, args.pile_steps)
    if rank == 0 and world == 1 and not args.no_box:
        # the box-drop configuration as stated (Coulomb friction 0.5 / 0.4)
        line["box_drop_configured"] = box_drop_rate(local)
    if rank == 0 and world == 1 and not args.no_batched:
        # batched scenes: 64 scenes in one system, autotuned, replayed as a
        # CUDA graph, against the same scenes stepped one after another
        from granular_gpu_gb300 import batch
        line["batched_scenes"] = batch.measure(64, frames=args.batched_frames, device=local)
        line["batched_scenes"]["unit"] = METRIC
    if rank == 0 and world == 1 and not args.no_learned:
        # learned warm start vs the plain sweeps, to the same residual, on a
        # held-out scene (device time of whole substeps, CUDA events): the
        # residual the configuration names (1e-3 r) and a looser one (1e-2 r)
        from granular_gpu_gb300 import learn
        mlp = learn.load_mlp(device=local)
        runs = {}
        for tol, frames, cap in ((1e-3, args.learned_frames, 2000), (1e-2, 150, 250)):
            ev = learn.evaluate(mlp, seeds=(101,), frames=frames, tol=tol, max_sweeps=cap, device=local)
            sc = ev["scenes"][0]
            runs[tol] = {
                "time_ratio": ev["time_ratio"], "sweep_ratio": ev["sweep_ratio"], "target_ratio": 0.6,
                "plain_ms": ev["plain_ms"], "learned_ms": ev["learned_ms"], "plain_sweeps": ev["plain_sweeps"],
                "learned_sweeps": ev["learned_sweeps"], "max_sweeps": cap,
                "plain_capped_frames": sc["plain_capped_frames"], "learned_capped_frames": sc["learned_capped_frames"],
                "residual": f"mean penetration over contacts <= {tol:g} r, checked before every Jacobi sweep "
                            f"(cap {cap} sweeps; a capped plain frame stops short, which favours the plain solver)",
                "scene": f"block 0.6x0.4x0.6 of {sc['particles']} particles (r=0.005, spacing 2r) dropped 0.02 onto "
                         f"the floor, Coulomb friction 0.5 / 0.4, held-out seed {sc['seed']}, {frames} substeps "
                         f"of 1/240 s"}
        mlp.close()
        line["learned_warm_start"] = dict(runs[1e-3])
        line["learned_warm_start"]["at_1e-2_r"] = runs[1e-2]
        line["learned_warm_start"]["network"] = ("48-64-64-3 MLP, BF16 tcgen05 kernels, trained on 2,000 solver frames "
                                                 "solved to 1e-3 r, Coulomb friction drawn U[0.3, 0.7] "
                                                 "(granular_gpu_gb300/weights/warm_start_mlp.npy)")
    if rank == 0 and world == 1 and not args.no_cpu:
        cv, threads, _ = cpu_sample(steps=args.cpu_steps, warmup=1)
        line["cpu_baseline"] = {"value": cv, "unit": METRIC, "cores": threads, "kind": "port",
                                "sample": SAMPLE_NOTE + f", {args.cpu_steps} timed substeps, FP64 build"}
        line["fp64_error"] = fp64_error(local)
    sysg.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist_on:
        tdist.destroy_process_group()
    return 0


def run_profile_window(args):
    """Steps the column to the headline window, then runs --steps substeps
    between cudaProfilerStart and cudaProfilerStop (for `ncu
    --profile-from-start off`), and prints the library's per-class CUDA-event
    times of those substeps as one JSON line.  No timing line of the
    benchmark; a number taken under a profiler is not one."""
    import torch
    import granular_gpu_gb300 as gg
    from granular_gpu_gb300 import workloads
    counts = tuple(int(c) for c in args.counts.split(","))
    desc = workloads.column_collapse(counts=counts, seed=42, constants=args.constants)
    if args.nlist_skin is not None:
        desc["params"].nlist_skin = args.nlist_skin * 0.002
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=0)
    start = args.window_start if args.window_start is not None else WINDOW_START
    if start > 1:
        s.step(start - 1)
    s.synchronize()
    torch.cuda.synchronize()
    s.profile_begin()
    torch.cuda.profiler.start()
    n0 = s.size()
    s.step(args.steps)
    s.synchronize()
    torch.cuda.profiler.stop()
    prof = s.profile_end()
    out = {"workload": f"column collapse {counts}, {args.constants} constants", "substeps": args.steps,
           "window_start": start, "particles": n0, "ms_per_substep": {
               k: round(v["ms"] / args.steps, 4) for k, v in prof.items() if isinstance(v, dict) and v["launches"]},
           "list_builds": prof.get("_nlist_rebuilds"), "kernel_launches": prof.get("_kernel_launches")}
    s.close()
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["mine", "reference"], default="mine")
    ap.add_argument("--cpu-steps", type=int, default=4)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-pile", action="store_true")
    ap.add_argument("--no-box", action="store_true", help="skip the box-drop configuration (Coulomb friction)")
    ap.add_argument("--no-scaled", action="store_true")
    ap.add_argument("--pile-steps", type=int, default=60)
    ap.add_argument("--batched-frames", type=int, default=10)
    ap.add_argument("--learned-frames", type=int, default=80,
                    help="substeps of the learned-warm-start comparison at 1e-3 r")
    ap.add_argument("--counts", default="128,256,256",
                    help="column lattice x,y,z (the benchmark workload is 128,256,256)")
    ap.add_argument("--math-mode", type=int, default=0)
    ap.add_argument("--nlist-skin", type=float, default=None,
                    help="contact-list skin in radii of 0.002 (default: a tenth of the cell length; "
                         "0 turns the lists off)")
    ap.add_argument("--profile-window", action="store_true",
                    help="profiling driver: step to the window, run --steps substeps between "
                         "cudaProfilerStart/Stop, print per-class times (no benchmark line)")
    ap.add_argument("--constants", choices=["reference", "scaled"], default="reference",
                    help="with --profile-window: the reference's length constants or them scaled by r/0.01")
    ap.add_argument("--window-start", type=int, default=None,
                    help="with --profile-window: first profiled substep (default: the headline window's)")
    args = ap.parse_args()
    if args.profile_window:
        import __graft_entry__
        __graft_entry__.build()
        return run_profile_window(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        # only the reference's kernels (prebuilt cubins where no checkout is
        # present); this library is not built or loaded in this arm
        from oracle import ref_cuda_build
        ref_cuda_build.build()
        return run_reference(args)
    import __graft_entry__
    __graft_entry__.build()
    return run_mine(args)


if __name__ == "__main__":
    sys.exit(main())
