"""Learned warm start: training data from the plain solver, training with
the library's tensor-core kernels, and the time-to-residual evaluation.

Scenes follow the adaptive-pile configuration's style without merge/split or
upsampling: a jittered block of particles of radius r = 0.005 (lattice
spacing 2r) released just above the floor of a box, substeps of dt = 1/240,
Coulomb friction with a static coefficient drawn U[0.3, 0.7] (the configured
mode: kinetic 0.8 of it, the box faces as analytic walls), and Jacobi sweeps
until the mean penetration over contacts is at most 1e-3 r
(gg_params.target_residual), or a cap on the sweeps is reached.  A frame is
one substep.  `python -m granular_gpu_gb300.learn train` (defaults: 8
scenes of 250 frames solved to 1e-3 r with at most 2,000 sweeps a frame)
makes the shipped weights.  The network is trained on the correction the
plain sweeps reach in each frame (recorded by the library with
gg_params.warm_start = 2) and evaluated on held-out seeds by Jacobi sweeps
and device time to the same residual, with and without the warm start,
from the same initial state.  `--law cap` runs the same with the
reference's contact law instead (friction as its tangential cap).
"""
import math
import os

import numpy as np

from . import GranularSystem, Mlp, abi, workloads
from .abi import FIELD_FEATURES, FIELD_WARM_TARGET

R = 0.005
DT = 1.0 / 240.0
TOL = 1e-3 * R


def pile_scene(seed: int, dims=(0.5, 0.5, 0.5), friction_cap: float = 0.5, r: float = R, drop: float = 0.02,
               target_residual: float = TOL, max_sweeps: int = 200, warm_start: int = 0, scale: float = 1.0,
               law: str = "coulomb"):
    """A jittered block (dims in metres, spacing 2r, jitter +-0.05r) centred
    in a box and released `drop` above the floor walls.  law="coulomb" (the
    default): the configured mode's Coulomb friction with mu_static =
    `friction_cap` and mu_kinetic = 0.8 of it, the box faces as analytic
    walls, Jacobi sweeps only; law="cap": the reference's contact law with
    `friction_cap` as its tangential cap, 3 stabilisation sweeps first."""
    L = np.float32(workloads.CELL_PER_RADIUS * r)
    counts = [max(2, int(round(d / (2 * r)))) for d in dims]
    side = max(1.0, 1.2 * max(counts[0], counts[2]) * 2 * r)
    height = max(1.0, 2.5 * counts[1] * 2 * r)
    space = (side, height, side)
    walls, cs = workloads.box_walls(space, L)
    floor = float(walls[:, 1].min())
    span = [(c - 1) * 2 * r for c in counts]
    origin = (side / 2 - span[0] / 2, floor + 0.01 * (r / 0.01) + r + drop, side / 2 - span[2] / 2)
    p = workloads.lattice(counts, 2 * r, origin, 0.05 * r, seed)
    params = workloads.scaled_params(r, iters=5)
    params.friction_cap = float(friction_cap)
    params.upsample_enabled = 0
    params.merge_enabled = 0
    params.target_residual = float(target_residual)
    params.max_sweeps = int(max_sweeps)
    params.warm_start = int(warm_start)
    params.warm_start_scale = float(scale)
    if law == "coulomb":
        workloads.configure(params, friction_cap, 0.8 * friction_cap, workloads.box_planes(space))
    elif law != "cap":
        raise ValueError(law)
    desc = workloads._desc(p, walls, None, space, L, cs, DT, (0.0, -9.81, 0.0), workloads.density_for_radius(r),
                           0, params, skip=True)
    return desc


def draw_scene(rng, **kw):
    """Block dimensions U[0.3, 0.8] m and friction U[0.3, 0.7] (the static
    Coulomb coefficient; with law="cap" the contact kernel's friction cap,
    0.8 in the reference)."""
    dims = tuple(float(rng.uniform(0.3, 0.8)) for _ in range(3))
    return pile_scene(int(rng.integers(1 << 30)), dims=dims, friction_cap=float(rng.uniform(0.3, 0.7)), **kw)


def collect(descs, frames: int, per_frame: int, device: int = 0, seed: int = 0, every: int = 1):
    """Runs each scene `frames` substeps with recording on and returns
    (features int16 n x 48, targets float32 n x 3) as torch CUDA tensors,
    `per_frame` random particles of every `every`-th frame."""
    import torch
    rng = np.random.default_rng(seed)
    X, T = [], []
    for d in descs:
        d = dict(d)
        d["params"].warm_start = 2
        s = GranularSystem(**workloads.system_kwargs(d), device=device)
        s.set_warm_start(None)
        for f in range(frames):
            s.step(1)
            if f % every:
                continue
            s.synchronize()
            n = s.size()
            fptr, fn, _ = s.device_ptr(FIELD_FEATURES)
            tptr, _, _ = s.device_ptr(FIELD_WARM_TARGET)
            feat = _view(fptr, (n, 48), torch.int16)
            targ = _view(tptr, (n, 3), torch.float32)
            idx = torch.as_tensor(rng.choice(n, min(per_frame, n), replace=False), device="cuda")
            X.append(feat.index_select(0, idx).clone())
            T.append(targ.index_select(0, idx).clone())
        s.close()
    return torch.cat(X).contiguous(), torch.cat(T).contiguous()


def _view(ptr: int, shape, dtype):
    """A torch tensor aliasing device memory the library owns."""
    import torch
    nbytes = int(np.prod(shape)) * torch.empty(0, dtype=dtype).element_size()

    class _Array:
        __cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (int(ptr), False),
                                    "version": 3}

    return torch.as_tensor(_Array(), device="cuda").view(dtype).view(*shape)


def train(mlp: Mlp, X, T, steps: int = 3000, batch: int = 16384, lr: float = 2e-3, seed: int = 0,
          log_every: int = 0):
    """Mini-batch Adam with the library's training kernel; returns the
    loss curve (one value per step)."""
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    n = X.shape[0]
    losses = []
    for k in range(steps):
        idx = torch.randint(0, n, (min(batch, n),), device="cuda", generator=g)
        xb = X.index_select(0, idx).contiguous()
        tb = T.index_select(0, idx).contiguous()
        lr_k = lr * 0.5 * (1.0 + math.cos(math.pi * k / steps))
        losses.append(mlp.train_step(xb, tb, xb.shape[0], lr=lr_k))
        if log_every and k % log_every == 0:
            print(f"step {k}: loss {losses[-1]:.4g}", flush=True)
    return losses


def run_scene(desc, frames: int, mlp=None, device: int = 0):
    """Device milliseconds, Jacobi sweeps and final residual of each frame
    of a scene in residual mode (warm start on when `mlp` is given)."""
    import torch
    d = dict(desc)
    d["params"].warm_start = 1 if mlp is not None else 0
    s = GranularSystem(**workloads.system_kwargs(d), device=device)
    if mlp is not None:
        s.set_warm_start(mlp)
    stream = torch.cuda.ExternalStream(s.stream, device=device)
    ms, sweeps, res = [], [], []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(frames):
        e0.record(stream)
        s.step(1)
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
        st = s.stats()
        sweeps.append(st["last_sweeps"])
        res.append(st["last_residual"])
    s.close()
    return np.array(ms), np.array(sweeps), np.array(res)


WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "warm_start_mlp.npy")
EVAL_DIMS = (0.6, 0.4, 0.6)  # the adaptive-pile configuration's block


def load_mlp(path: str = WEIGHTS, device: int = 0) -> Mlp:
    """The network with the trained parameters of `path`."""
    m = Mlp(device=device, seed=0)
    m.set_params(np.load(path).astype(np.float32))
    return m


def evaluate(mlp: Mlp, seeds=(101, 102), frames: int = 150, dims=EVAL_DIMS, tol: float = 1e-2,
             friction_cap: float = 0.5, device: int = 0, max_sweeps: int = 250, law: str = "coulomb") -> dict:
    """Plain vs warm-started residual-mode runs of held-out scenes from the
    same initial state: device ms and Jacobi sweeps summed over the frames,
    and the frames that reached the residual within the sweep cap."""
    out = {"tolerance_r": tol, "frames": frames, "max_sweeps": max_sweeps, "scenes": []}
    tp = tl = sp = sl = 0.0
    for seed in seeds:
        d = pile_scene(seed, dims=dims, friction_cap=friction_cap, target_residual=tol * R, max_sweeps=max_sweeps,
                       law=law)
        msp, swp, rp = run_scene(d, frames, device=device)
        msl, swl, rl = run_scene(d, frames, mlp=mlp, device=device)
        out["scenes"].append({"seed": seed, "particles": d["n_particles"], "plain_ms": float(msp.sum()),
                              "learned_ms": float(msl.sum()), "plain_sweeps": int(swp.sum()),
                              "learned_sweeps": int(swl.sum()),
                              "plain_capped_frames": int((swp >= max_sweeps).sum()),
                              "learned_capped_frames": int((swl >= max_sweeps).sum()),
                              "plain_final_residual_r": float(rp[-1] / R), "learned_final_residual_r": float(rl[-1] / R)})
        tp += msp.sum()
        tl += msl.sum()
        sp += swp.sum()
        sl += swl.sum()
    out.update(plain_ms=float(tp), learned_ms=float(tl), time_ratio=float(tl / tp), plain_sweeps=int(sp),
               learned_sweeps=int(sl), sweep_ratio=float(sl / sp))
    return out


def main(argv=None):
    import argparse
    import json
    import time
    ap = argparse.ArgumentParser(description="train or evaluate the learned warm start")
    ap.add_argument("cmd", choices=["train", "evaluate", "bench"],
                    help="train: collect and train; evaluate: plain vs warm start; "
                         "bench: time the network's kernels on random features")
    ap.add_argument("--rows", type=int, default=1 << 22, help="feature rows (bench)")
    ap.add_argument("--scenes", type=int, default=8)
    ap.add_argument("--frames", type=int, default=250, help="frames per training scene (train) or per run (evaluate)")
    ap.add_argument("--per-frame", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--batch", type=int, default=16384)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--tol", type=float, default=1e-3, help="mean-penetration tolerance in radii")
    ap.add_argument("--max-sweeps", type=int, default=2000, help="cap on the Jacobi sweeps of a frame")
    ap.add_argument("--weights", default=WEIGHTS)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--eval-seeds", default="101,102")
    ap.add_argument("--law", choices=["cap", "coulomb"], default="coulomb",
                    help="contact law of the scenes: Coulomb friction (configured mode), or the reference's "
                         "friction cap")
    a = ap.parse_args(argv)
    if a.cmd == "train":
        rng = np.random.default_rng(a.seed)
        descs = [draw_scene(rng, target_residual=a.tol * R, max_sweeps=a.max_sweeps, law=a.law)
                 for _ in range(a.scenes)]
        t0 = time.time()
        X, T = collect(descs, frames=a.frames, per_frame=a.per_frame, seed=a.seed)
        t1 = time.time()
        m = Mlp(seed=a.seed + 1)
        losses = train(m, X, T, steps=a.steps, batch=a.batch, lr=a.lr, seed=a.seed)
        t2 = time.time()
        os.makedirs(os.path.dirname(os.path.abspath(a.weights)), exist_ok=True)
        np.save(a.weights, m.get_params())
        print(json.dumps({"frames": a.scenes * a.frames, "samples": int(X.shape[0]),
                          "scene_particles": [d["n_particles"] for d in descs],
                          "collect_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2),
                          "loss_first": losses[0], "loss_last": float(np.mean(losses[-100:])),
                          "target_variance": float(T.var().item()), "weights": a.weights}))
    elif a.cmd == "evaluate":
        m = load_mlp(a.weights)
        seeds = tuple(int(s) for s in a.eval_seeds.split(","))
        print(json.dumps(evaluate(m, seeds=seeds, frames=a.frames, tol=a.tol, max_sweeps=a.max_sweeps, law=a.law)))
    else:
        print(json.dumps(bench_kernels(a.rows, seed=a.seed)))
    return 0


def bench_kernels(n: int, seed: int = 0, reps: int = 10) -> dict:
    """Device time of the network's forward and gradient kernels over n
    random bf16 feature rows (three untimed forward + training passes
    first), with the work they issue to the tensor cores."""
    import torch
    rng = np.random.default_rng(seed)
    x = rng.normal(0, 1.5, (n, Mlp.N_FEATURES)).astype(np.float32)
    x[:, 0] = 1.0
    bits = (x.view(np.uint32) + 0x7FFF + ((x.view(np.uint32) >> 16) & 1)) >> 16  # round to bf16
    xd = torch.as_tensor(bits.astype(np.uint16).view(np.int16), device="cuda")
    td = torch.as_tensor(rng.normal(0, 1, (n, Mlp.N_OUT)).astype(np.float32), device="cuda")
    yd = torch.zeros((n, Mlp.N_OUT), device="cuda")
    m = Mlp(seed=seed + 1)
    for _ in range(3):
        m.forward(xd, yd, n)
        m.train_step(xd, td, n, lr=1e-3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    fwd = timed(lambda: m.forward(xd, yd, n))
    grd = timed(lambda: m.gradient(xd, td, n))
    m.close()
    flops_f = 2 * n * (48 * 64 + 64 * 64 + 64 * 16)
    flops_g = flops_f + 2 * n * (16 * 64 + 64 * 64) + 2 * n * 128 * (16 + 64 + 64)
    return {"rows": n, "forward_ms": fwd, "forward_feature_gbs": n * 96 / fwd / 1e6,
            "forward_tflops": flops_f / fwd / 1e9, "gradient_ms": grd, "gradient_tflops": flops_g / grd / 1e9}


if __name__ == "__main__":
    raise SystemExit(main())
