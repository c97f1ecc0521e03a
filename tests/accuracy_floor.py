"""Binary32 storage floor of the served FP32 form's accuracy (test
infrastructure; CPU only, uses the oracle).

For each sampled request of the served benchmark's stream, two oracle runs
from the same initial condition: the plain binary64 run (bit-identical to the
reference), and a run in the same binary64 arithmetic whose conservative
state is rounded to binary32 after every step, stored as the offset from the
background the service uses (the medians of the initial density and total
energy over at most 64 x 64 sampled cells) -- fv2d_oracle_round_cons_f32.
The L1 relative density and pressure differences between the two, at the
checkpoints bench.py --served-accuracy samples the service at, are the error
that binary32 storage of the state causes by itself, before any binary32
arithmetic: the floor the service's own error is read against.

    python tests/accuracy_floor.py [--every 16] [--nmax 1024] > floor.jsonl
    python tests/accuracy_floor.py --configs > floor_configs.jsonl

--configs: the reduced Kelvin-Helmholtz and Rayleigh-Taylor set-ups of
bench.py --fp32-configs-only --fp32-configs-reduced, at t = tend k / 8 (each
run stops at the first t at or past each of those times).
"""
import argparse
import ctypes as C
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))

import fv2d_testlib as T  # noqa: E402


def service_background(u, nx, ny):
    """The background the service stores offsets from (serve.cu,
    background()): upper medians of rho and E over the cells (sy/2 + k sy,
    sx/2 + l sx), sx = max(1, Nx / 64), rounded to binary32."""
    sx, sy = max(1, nx // 64), max(1, ny // 64)
    sub = u[sy // 2::sy, sx // 2::sx]
    out = np.zeros(4)
    for k in (0, 3):
        v = np.sort(sub[..., k].ravel())
        out[k] = float(np.float32(v[len(v) // 2]))
    return out


def floor_curve(req, points):
    lib = T.oracle_lib()
    lib.fv2d_oracle_round_cons_f32.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    p = req["params"]
    a = T.Oracle(p)
    a.init_problem(req["problem"])
    b = T.Oracle(p)
    b.init_problem(req["problem"])
    bg = service_background(b.get_cons(), p.Nx, p.Ny)
    bgp = bg.ctypes.data_as(C.POINTER(C.c_double))
    lib.fv2d_oracle_round_cons_f32(b.h, bgp)

    def l1(x, y, k):
        return float(np.sum(np.abs(x[..., k] - y[..., k])) / np.sum(np.abs(y[..., k])))
    curve, done = [], 0
    for n in points:
        for _ in range(n - done):
            a.update(a.compute_dt()[0])
            b.update(b.compute_dt()[0])
            lib.fv2d_oracle_round_cons_f32(b.h, bgp)
        done = n
        qa, qb = a.get_prim(), b.get_prim()
        curve.append([n, l1(qb, qa, 0), l1(qb, qa, 3)])
    return curve, bg


def floor_curve_time(problem, p, tend, n=8):
    lib = T.oracle_lib()
    lib.fv2d_oracle_round_cons_f32.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
    a = T.Oracle(p)
    a.init_problem(problem)
    b = T.Oracle(p)
    b.init_problem(problem)
    bg = service_background(b.get_cons(), p.Nx, p.Ny)
    bgp = bg.ctypes.data_as(C.POINTER(C.c_double))
    lib.fv2d_oracle_round_cons_f32(b.h, bgp)
    ta = tb = 0.0
    na = nb = 0
    curve = []
    for k in range(1, n + 1):
        tk = tend * k / n
        while ta + p.epsilon < tk:
            d = a.compute_dt()[0]
            a.update(d)
            ta += d
            na += 1
        while tb + p.epsilon < tk:
            d = b.compute_dt()[0]
            b.update(d)
            lib.fv2d_oracle_round_cons_f32(b.h, bgp)
            tb += d
            nb += 1
        qa, qb = a.get_prim(), b.get_prim()
        l1 = [float(np.sum(np.abs(qb[..., f] - qa[..., f])) / np.sum(np.abs(qa[..., f]))) for f in (0, 3)]
        curve.append({"t": tk, "steps_fp64": na, "steps_floor": nb, "l1_rho": l1[0], "l1_p": l1[1]})
    return curve


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--every", type=int, default=16)
    ap.add_argument("--nmax", type=int, default=1024)
    ap.add_argument("--configs", action="store_true")
    args = ap.parse_args()
    import bench
    if args.configs:
        import fv2d_gb300 as fv
        T.oracle_lib().fv2d_oracle_set_threads(os.cpu_count() or 1)
        for name, (problem, tend, p) in bench.fp32_configs(fv, reduced=True).items():
            t0 = time.perf_counter()
            curve = floor_curve_time(problem, p, tend)
            print(json.dumps({"config": name, "curve": curve, "seconds": time.perf_counter() - t0}), flush=True)
        return
    from fv2d_gb300.serve import stream_requests
    reqs = stream_requests()
    T.oracle_lib().fv2d_oracle_set_threads(os.cpu_count() or 1)
    for i in range(0, len(reqs), args.every):
        r = reqs[i]
        if r["N"] > args.nmax:
            continue
        t0 = time.perf_counter()
        curve, bg = floor_curve(r, bench.checkpoints(r["steps"]))
        print(json.dumps({"i": i, "kind": r["kind"], "N": r["N"], "steps": r["steps"], "floor_l1_rho": curve[-1][1],
                          "floor_l1_p": curve[-1][2], "curve": curve, "background": [bg[0], bg[3]],
                          "seconds": time.perf_counter() - t0}), flush=True)


if __name__ == "__main__":
    main()
