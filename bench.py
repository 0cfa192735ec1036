"""Benchmark: particle-substeps/s of the column-collapse workload on GB300.

A "step" is one substep of the reference's GranularSystem::step (grid
build, 3 stabilisation + 4 Jacobi sweeps, finalize, upsampling of 4 render
points per particle, surface detection and merge/split on the integer
ledger) over 8,388,608 particles resident in HBM.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]

N > 1 runs N independent replicas (one per rank, launched by torchrun); the
path has no exchange step.  `--impl reference` times the CPU restatement of
the reference's path (the reference itself is CUDA-only, it has no CPU
implementation) on a bounded sample of the same workload.
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
           "3+4 sweeps, merge/split to mass 8, 4 render points/particle)"
SAMPLE_COUNTS = (64, 64, 64)
SAMPLE_NOTE = "64x64x64 sub-lattice (262,144 particles) of the same column scene (same box, grid, walls, " \
              "parameters), one oracle substep per step"
# Algorithmic (compulsory) bytes per unit of each kernel class, with FP32
# float3 state and neighbour re-reads assumed to hit in cache: the roofline
# is reported for whichever class takes the most time in the timed region.
ALGO_BYTES = {
    "sweep": (28, "particle", "read x* and radius 16 B, write x* 12 B"),
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
    desc = workloads.column_collapse(counts=SAMPLE_COUNTS)
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
    the bounded sample: max |x - x_fp64| in units of r and max |v - v_fp64|.
    (After a second grid build the two sort particles near cell faces
    differently, so particles compare index by index after one substep.)"""
    import granular_gpu_gb300 as gg
    from granular_gpu_gb300 import abi, workloads
    from oracle import oracle as orc
    desc = workloads.column_collapse(counts=SAMPLE_COUNTS)
    s = gg.GranularSystem(**workloads.system_kwargs(desc), device=device)
    o = orc.OracleSystem(desc, fp64=True)
    if s.size() != o.size():
        out = {"unavailable": f"particle counts differ ({s.size()} vs {o.size()})"}
    else:
        r = 0.002
        dx = np.abs(s.read(gg.FIELD_POS).astype(np.float64) - o.read(abi.FIELD_POS).astype(np.float64)).max()
        dv = np.abs(s.read(gg.FIELD_VEL).astype(np.float64) - o.read(abi.FIELD_VEL).astype(np.float64)).max()
        out = {"pos_max_abs_r": float(dx / r), "vel_max_abs": float(dv), "substeps": 1,
               "sample": "64x64x64 sub-lattice of the column scene, FP32 CUDA math against the FP64 build"}
    s.close()
    o.close()
    return out


def run_reference(args):
    rank, world, _ = _dist()
    if rank != 0:
        return 0
    value, threads, dt = cpu_sample(args.steps, args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": {"workload": WORKLOAD, "sample": SAMPLE_NOTE},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                         "sample": SAMPLE_NOTE},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
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
    desc = workloads.column_collapse(counts=counts, seed=42 + rank)
    if args.math_mode:
        desc["params"].math_mode = args.math_mode
    if args.nlist_skin is not None:
        desc["params"].nlist_skin = args.nlist_skin * 0.002
    n0 = desc["n_particles"]
    sysg = gg.GranularSystem(**workloads.system_kwargs(desc), device=local)
    stream = torch.cuda.ExternalStream(sysg.stream, device=local)
    for _ in range(args.warmup):
        sysg.step(1)
    sysg.synchronize()

    def barrier():
        if dist_on:
            tdist.barrier()

    # ---- device-resident timed region
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sysg.profile_begin()
    units = 0
    ev0.record(stream)
    for _ in range(args.steps):
        units += sysg.size()
        sysg.step(1)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    prof = sysg.profile_end()
    launches = prof.pop("_kernel_launches")
    list_builds = prof.pop("_nlist_rebuilds")
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    ms_max, total_units = reduce_over_ranks(ms, units)
    value = total_units / (ms_max / 1000.0)

    # ---- end to end through the C ABI with pinned host buffers
    if args.no_e2e:
        args.steps_e2e = 0
    else:
        args.steps_e2e = args.steps
    n = sysg.size()
    nu = sysg.upsampled_size()
    hp = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    hv = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    hu = torch.empty((nu, 3), dtype=torch.float32, pin_memory=True).numpy()
    sysg.read(gg.FIELD_POS, out=hp)
    sysg.read(gg.FIELD_VEL, out=hv)
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e2e_units = 0
    h2d = d2h = 0
    for _ in range(args.steps_e2e):
        m = sysg.size()
        if hp.shape[0] != m:
            hp = torch.empty((m, 3), dtype=torch.float32, pin_memory=True).numpy()
            hv = torch.empty((m, 3), dtype=torch.float32, pin_memory=True).numpy()
            sysg.read(gg.FIELD_POS, out=hp)
            sysg.read(gg.FIELD_VEL, out=hv)
        sysg.write(gg.FIELD_POS, hp)
        sysg.write(gg.FIELD_VEL, hv)
        h2d += 2 * hp.nbytes
        e2e_units += m
        sysg.step(1)
        m = sysg.size()
        if hp.shape[0] != m:
            hp = torch.empty((m, 3), dtype=torch.float32, pin_memory=True).numpy()
            hv = torch.empty((m, 3), dtype=torch.float32, pin_memory=True).numpy()
        sysg.read(gg.FIELD_POS, out=hp)
        sysg.read(gg.FIELD_VEL, out=hv)
        sysg.read(gg.FIELD_POS, gg.SET_UPSAMPLED, out=hu)
        d2h += 2 * hp.nbytes + hu.nbytes
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_s_max, e2e_total = reduce_over_ranks(e2e_s, e2e_units)
    e2e_value = e2e_total / e2e_s_max if args.steps_e2e else None

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

    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD if counts == (128, 256, 256) else f"column collapse {counts}",
                   "particles": n0, "upsampled": desc["n_upsampled"],
                   "boundary": desc["n_boundary"], "cells": int(np.prod(desc["cell_size"])),
                   "l2": "inputs larger than L2 (about 1.9 GB of particle state per step)",
                   "parallelism": f"replicas x{world}"},
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
                "d2h_bytes_per_step": d2h // max(args.steps, 1)},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if rank == 0 and world == 1 and not args.no_pile:
        # the adaptive-pile configuration: 262,144 particles of r = 0.005 on the
        # floor of a box with a 30-degree ramp, merge/split to mass 8 on the
        # integer ledger, 4 render points per particle; timed after 100
        # substeps (merges under way)
        line["adaptive_pile"] = pile_rate(local, args.pile_steps)
    if rank == 0 and world == 1 and not args.no_batched:
        # batched scenes: 64 scenes in one system, autotuned, replayed as a
        # CUDA graph, against the same scenes stepped one after another
        from granular_gpu_gb300 import batch
        line["batched_scenes"] = batch.measure(64, frames=args.batched_frames, device=local)
        line["batched_scenes"]["unit"] = METRIC
    if rank == 0 and world == 1 and not args.no_learned:
        # learned warm start vs the plain sweeps, to the same residual, on a
        # held-out scene (device time of whole substeps, CUDA events)
        from granular_gpu_gb300 import learn
        mlp = learn.load_mlp(device=local)
        ev = learn.evaluate(mlp, seeds=(101,), frames=args.learned_frames, device=local)
        mlp.close()
        sc = ev["scenes"][0]
        line["learned_warm_start"] = {
            "time_ratio": ev["time_ratio"], "sweep_ratio": ev["sweep_ratio"], "target_ratio": 0.6,
            "plain_ms": ev["plain_ms"], "learned_ms": ev["learned_ms"], "plain_sweeps": ev["plain_sweeps"],
            "learned_sweeps": ev["learned_sweeps"], "plain_capped_frames": sc["plain_capped_frames"],
            "learned_capped_frames": sc["learned_capped_frames"],
            "residual": "mean penetration over contacts <= 1e-2 r, checked before every Jacobi sweep (cap 250); "
                        "the plain sweeps do not bring the max penetration to 1e-3 r on a pile",
            "scene": f"block 0.6x0.4x0.6 of {sc['particles']} particles (r=0.005, spacing 2r) dropped 0.02 onto "
                     f"the floor, held-out seed {sc['seed']}, {args.learned_frames} substeps of 1/240 s",
            "network": "48-64-64-3 MLP, BF16 tcgen05 kernels, trained on 2,000 solver frames "
                       "(granular_gpu_gb300/weights/warm_start_mlp.npy)"}
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
    ap.add_argument("--pile-steps", type=int, default=60)
    ap.add_argument("--batched-frames", type=int, default=10)
    ap.add_argument("--learned-frames", type=int, default=150)
    ap.add_argument("--counts", default="128,256,256",
                    help="column lattice x,y,z (the benchmark workload is 128,256,256)")
    ap.add_argument("--math-mode", type=int, default=0)
    ap.add_argument("--nlist-skin", type=float, default=None,
                    help="contact-list skin in radii of 0.002 (default: a tenth of the cell length; "
                         "0 turns the lists off)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    import __graft_entry__
    __graft_entry__.build()
    if args.impl == "reference":
        return run_reference(args)
    return run_mine(args)


if __name__ == "__main__":
    sys.exit(main())
