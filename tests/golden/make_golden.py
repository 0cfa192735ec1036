"""Generates the known-answer vectors in tests/golden/known_answers.json.

The reference ships no tests or fixtures for its substep path, and its CUDA
build cannot run here.  These vectors restate the reference's arithmetic
for tiny, hand-checkable cases in scalar float32 Python, independently of
the C oracle, so the oracle can be pinned against them:

  grid      keys of hand-placed points (CUDAFunctions.cuh:71-107), the
            stable sort order and the cell start table (GranularSystem.cu:65-173)
  pair      two overlapping unit masses, no gravity, one reference step of
            3 stabilisation + 5 Jacobi sweeps (Solver.cu:309-513): each
            sweep moves each particle by w (r_i + r_j - d) / n with n = 2
  wall      one particle overlapping one wall particle (Solver.cu:272-307)
  damping   final_velocity_functor cases (Solver.cu:193-248)
  upsample  one render point near one coarse particle (Solver.cu:1244-1369)

Run:  python tests/golden/make_golden.py
"""
import json
import math
import os

import numpy as np

F = np.float32
HERE = os.path.dirname(os.path.abspath(__file__))


def f(x):
    return F(x)


def grid_case():
    L = F(0.5)
    cs = (4, 3, 5)
    C = cs[0] * cs[1] * cs[2]
    pts = [(0.1, 0.1, 0.1), (0.6, 0.1, 0.1), (1.99, 1.49, 2.49), (2.0, 0.0, 0.0), (-0.01, 0.2, 0.2),
           (0.5, 0.5, 0.5), (0.1, 0.1, 0.1), (0.74, 0.26, 0.26), (0.6, 0.1, 0.1), (1.0, 1.0, 1.0)]
    keys = []
    for p in pts:
        c = [int(math.floor(F(p[k]) / L)) for k in range(3)]
        inside = all(0 <= c[k] < cs[k] for k in range(3))
        keys.append(((c[0] * cs[1]) + c[1]) * cs[2] + c[2] if inside else C)
    order = sorted(range(len(pts)), key=lambda i: (keys[i], i))
    sk = [keys[i] for i in order]
    counts = [0] * (C + 1)
    for k in keys:
        counts[k] += 1
    start, run = [], 0
    for c in counts:
        start.append(run)
        run += c
    return {"cell_size": cs, "cell_length": float(L), "points": pts, "keys": keys, "sorted_keys": sk,
            "perm": order, "cell_start": start}


def radius_contact(m, rho):
    # cbrtf((3*m) / (4*pi*(int)density)) with double pi (Solver.cu:320)
    return F(np.cbrt(F(float(F(3) * F(m)) / (4.0 * math.pi * float(int(rho))))))


def norm3(a, b, c):
    return F(math.sqrt(float(a) ** 2 + float(b) ** 2 + float(c) ** 2))


def pair_case():
    rho = 238732.4146
    r = radius_contact(1.0, rho)
    y = F(0.5)
    x0 = [F(0.5), y, F(0.5)]
    x1 = [F(0.515), y, F(0.5)]
    # scaled masses are equal (same height): inverse masses equal
    sm = F(F(1.0) * F(np.exp(F(-y))))
    inv = F(F(1.0) / sm)
    pos = [list(x0), list(x1)]
    xs = [list(x0), list(x1)]
    for it in range(8):
        deltas = []
        for i, j in ((0, 1), (1, 0)):
            p12 = [F(xs[i][k] - xs[j][k]) for k in range(3)]
            inv_sum = F(1.0 / float(F(inv + inv)))
            dis = norm3(*p12)
            mag = F(F(r + r) - dis)
            assert mag >= 0
            t = F(mag / dis)
            dpi = [F(F(F(-inv_sum * inv) * t) * p12[k]) for k in range(3)]
            dpj = [F(F(F(inv_sum * inv) * t) * p12[k]) for k in range(3)]
            dpij = [F(dpi[k] - dpj[k]) for k in range(3)]
            w = F(inv_sum * inv)
            deltas.append([F(F(0) - F(w * dpij[k])) for k in range(3)])
        for i in range(2):
            inc = [F(deltas[i][k] / F(2)) for k in range(3)]
            if it < 3:
                pos[i] = [F(pos[i][k] + inc[k]) for k in range(3)]
            xs[i] = [F(xs[i][k] + inc[k]) for k in range(3)]
    dt = F(0.002)
    dt_inv = F(F(1) / dt)
    vel = []
    for i in range(2):
        v = [F(dt_inv * F(xs[i][k] - pos[i][k])) for k in range(3)]
        speed = F(math.sqrt(float(F(F(F(v[0] * v[0]) + F(v[1] * v[1])) + F(v[2] * v[2])))))
        if speed < F(0.01):
            v = [F(0), F(0), F(0)]
        vel.append(v)
    return {"density": rho, "dt": float(dt), "radius": float(r), "x0": [float(v) for v in x0],
            "x1": [float(v) for v in x1],
            "pos": [[float(v) for v in p] for p in xs], "vel": [[float(v) for v in p] for p in vel],
            "contacts": [1, 1], "num_constraints": [2, 2]}


def wall_case():
    rho = 238732.4146
    r = radius_contact(1.0, rho)
    rb = max(r, F(0.01))
    B = 0.01 + float(rb)
    b = [F(0.5), F(0.5), F(0.5)]
    x = [F(0.5), F(0.515), F(0.5)]
    pos, xs = list(x), list(x)
    for it in range(8):
        p12 = [F(xs[k] - b[k]) for k in range(3)]
        dis = norm3(*p12)
        mag = F(float(dis) - B)
        if mag < 0:
            dpi = [F(F(mag / dis) * p12[k]) for k in range(3)]
            dp = [F(F(0) - dpi[k]) for k in range(3)]
            n = 1
        else:
            dp, n = [F(0)] * 3, 0
        inc = [F(dp[k] / F(max(1, n))) for k in range(3)]
        if it < 3:
            pos = [F(pos[k] + inc[k]) for k in range(3)]
        xs = [F(xs[k] + inc[k]) for k in range(3)]
    return {"density": rho, "boundary": [float(v) for v in b], "x": [float(v) for v in x],
            "pos": [float(v) for v in xs], "separation": float(norm3(*[F(xs[k] - b[k]) for k in range(3)]))}


def damping_case():
    # one free particle, no gravity, initial velocity v0 along x:
    # x* = x + dt v0, v = (x* - x) / dt, then the damping of
    # final_velocity_functor (adaptive_last_step = 0)
    dt = F(0.002)
    out = []
    for v0 in (0.004, 0.5, 2.0, 25.0):
        x = F(0.3)
        xs = F(x + F(dt * F(v0)))
        v = F(F(F(1) / dt) * F(xs - x))
        speed = abs(v)
        if speed < F(0.01):
            r = F(0)
        elif speed > F(1.0):
            t = min(max(F(F(speed - F(1.0)) / F(F(10.0) - F(1.0))), F(0)), F(1))
            damping = F(F(0.99) + F(F(F(0.99) - F(0.99)) * t))
            fac = F(damping + F(F(F(1) - damping) * F(np.exp(F(-speed * F(0.1))))))
            r = F(v * fac)
        else:
            r = v
        out.append({"v0": v0, "x": float(xs), "velocity": float(r)})
    return {"dt": float(dt), "cases": out}


def upsample_case():
    # one render point at rest 0.02 from one coarse particle at rest
    r9 = F(493.8271605)
    p = [F(0.5), F(0.5), F(0.5)]
    q = [F(0.52), F(0.5), F(0.5)]
    d = [F(p[k] - q[k]) for k in range(3)]
    dis = F(math.sqrt(float(F(F(F(d[0] * d[0]) + F(d[1] * d[1])) + F(d[2] * d[2])))))
    t1 = F(F(1) - F(F(dis * dis) * r9))
    w = max(F(0), F(F(t1 * t1) * t1))
    wv = [F(F(w * F(0)) / w) for k in range(3)]
    alpha = max(F(0), F(F(1) - w))
    gdt = [F(F(0) * F(0.002)), F(F(-9.8) * F(0.002)), F(F(0) * F(0.002))]
    nv = [F(F(alpha * F(F(0) + gdt[k])) + F(F(F(1) - alpha) * wv[k])) for k in range(3)]
    up = [F(p[k] + F(nv[k] * F(0.002))) for k in range(3)]
    return {"point": [float(v) for v in p], "particle": [float(v) for v in q],
            "weight": float(w), "vel": [float(v) for v in nv], "pos": [float(v) for v in up]}


def main():
    data = {"grid": grid_case(), "pair": pair_case(), "wall": wall_case(), "damping": damping_case(),
            "upsample": upsample_case()}
    with open(os.path.join(HERE, "known_answers.json"), "w") as fh:
        json.dump(data, fh, indent=1)
    print("wrote known_answers.json")


if __name__ == "__main__":
    main()
