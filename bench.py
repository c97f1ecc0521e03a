#!/usr/bin/env python
"""Benchmark of the GB300 explicit hydro step (plain FP64 path).

Workload (headline configuration): Sedov blast, 2048 x 2048 cells on
[0,1]^2, rho = 1, u = v = 0, ambient p = 1e-5, E0 = 1 deposited as uniform
pressure in the cells within r0 = 0.02 of the centre, gamma = 1.4, PLM/minmod,
HLLC, CFL 0.8, reflecting walls, binary64.  Parameters are float-rounded the
way the reference's .ini reader returns them.  One bench step is one full
hydro iteration over the grid (dt reduction + fused update), computed on the
device from the previous state.

  value   cell-updates/s with the state resident in HBM: K iterations queued
          with fv2d_run_async, timed with CUDA events on the library's stream
          (the state, 402 MB, is larger than the 129 MB L2, so no flush).
  e2e     the same metric through the C-ABI with host buffers: per step
          fv2d_set_prim from page-locked host memory (read by the set-up
          kernel over the host link), fv2d_compute_dt, fv2d_update (which
          also writes the new state into a registered page-locked host
          mirror while it computes), fv2d_get_prim on that mirror.

`--impl reference` times the reference's own step code on the host cores (its
headers built with OpenMP over rows in place of Kokkos' dispatch, from the
sources staged into baseline/_ref), on the same workload; where those sources
are not staged, the CPU oracle (an OpenMP restatement of the reference's pass
structure, bit-exact with the reference's headers) stands in.

Launched as `python bench.py --gpus N --steps K --warmup W` (N = 1) or under
torch.distributed.run for N > 1: ranks run independent replicas (the step
has no exchange between simulations) and `value` sums them.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

NX = NY = 2048
BYTES_PER_CELL = 64  # read + write 4 x binary64 conservative state per cell-update
METRIC = "cell-updates/s"
WORKLOAD = "sedov_2048x2048_fp64_plain"


def workload_params(fv, n):
    f = fv.as_float32
    return fv.default_params(Nx=n, Ny=n, xmin=0.0, xmax=1.0, ymin=0.0, ymax=1.0, gamma0=f(1.4), CFL=f(0.8),
                             reconstruction=fv.PLM, riemann_solver=fv.HLLC, boundary_x=fv.BC_REFLECTING,
                             boundary_y=fv.BC_REFLECTING, time_stepping=fv.TS_EULER)


def max_over_ranks(x, dist=None, device="cpu"):
    """Maximum of x over the ranks of the default process group (x itself
    when there is none): the slowest replica sets the whole job's time."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, seconds_max):
    """Units processed by all replicas per second of the slowest one."""
    return world * units_per_rank / seconds_max


def config(n, steps):
    return {"workload": WORKLOAD, "grid": [n, n], "problem": "sedov", "scheme": "PLM-minmod + HLLC, Euler",
            "cfl": 0.8, "gamma": 1.4, "boundaries": "reflecting", "steps": steps,
            "l2": "state 402 MB (> 129 MB L2) streamed every step; no flush needed",
            "precision": "binary64, bit-identical to the reference"}


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def profile_figures():
    """Per-cell figures of the step kernel from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "step_fp64_plm_hllc_sedov.txt")
    out = {}
    if os.path.exists(path):
        for line in open(path):
            if ":" in line and line.split(":", 1)[0].strip() in (
                    "dram_bytes_per_cell", "fp64_pipe_ops_per_cell", "dram_bytes_per_launch_2048"):
                k, v = line.split(":", 1)
                try:
                    out[k.strip()] = float(v.split()[0])
                except ValueError:
                    pass
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.path = os.path.join("/tmp", f"fv2d_clocks_{os.getpid()}.csv")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(gpu_index), "-lms", "200"], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_reference_sim(n):
    """The CPU implementation of the step timed as the baseline, on the Sedov
    workload at n x n: the reference's own step code (its headers compiled
    with OpenMP over rows in place of Kokkos' dispatch, oracle/_ref, built
    from the staged reference sources) when that build is present, else the
    oracle port (an OpenMP restatement of the reference's pass structure,
    bit-identical to it).  Returns (compute_dt, update, kind, what, cores)."""
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import fv2d_testlib as T
    p = T.reference_params(Nx=n, Ny=n, gamma0=1.4, CFL=0.8, reconstruction=2, riemann_solver=1, boundary_x=1,
                           boundary_y=1)
    o = T.Oracle(p)
    o.init_problem("sedov")
    ncores = os.cpu_count() or 1
    T.oracle_lib().fv2d_oracle_set_threads(ncores)
    if T.ref_available(T.REF_OMP_SO):
        r = T.RefSim(p, lib_path=T.REF_OMP_SO)
        r.set_prim(o.get_prim())  # the Sedov initial condition (not one of the reference's problems)
        del o
        return (lambda: r.compute_dt(), r.update, "reference",
                "the reference's own step code (UpdateFunctor::update, ComputeDtFunctor::computeDt, consToPrim, "
                "checkNegatives from its headers) built -O3 with OpenMP over rows in place of Kokkos' dispatch", ncores)
    return (lambda: o.compute_dt()[0], o.update, "port",
            "oracle: OpenMP restatement of the reference pass structure, -O3 -ffp-contract=off (the reference's "
            "sources were not staged on this host)", T.oracle_lib().fv2d_oracle_get_threads())


def cpu_oracle_rate(n, steps_cap=500, budget_s=12.0):
    """CPU baseline cell-updates/s on a bounded sample of the workload: the
    same Sedov grid, as many iterations as fit about budget_s seconds (at
    most steps_cap), on all host cores."""
    cdt, upd, kind, what, cores = cpu_reference_sim(n)
    t0 = time.perf_counter()
    upd(cdt())
    one = time.perf_counter() - t0
    steps = max(1, min(steps_cap, int(budget_s / max(one, 1e-6))))
    t0 = time.perf_counter()
    for _ in range(steps):
        upd(cdt())
    el = time.perf_counter() - t0
    return {"value": n * n * steps / el, "unit": METRIC, "cores": cores, "kind": kind,
            "sample": f"sedov {n}x{n}, {steps} iterations after 1 warm-up; {what}", "seconds": el}


def run_served(fv, n_requests=512, rate=200.0, sample_every=16, budget=150e9, device=0, active_cells=8e6,
               single_launch=False):
    """The batched FP32 service on the seeded request stream: requests are
    submitted at their Poisson arrival times; every 16th request is also run
    alone through the plain FP64 path (bit-identical to the reference) for
    the time-to-solution and throughput comparison and the accuracy check."""
    from fv2d_gb300.serve import Server, stream_requests, config_name
    reqs = stream_requests(n=n_requests, rate=rate)
    sample = set(range(0, len(reqs), sample_every))
    srv = Server(budget_bytes=budget, device=device, autotune=True, active_cells=active_cells,
                 single_launch=single_launch)
    st0 = srv.stats()
    results, ids, keep = {}, {}, {}
    t_start = time.perf_counter()
    k = 0
    while k < len(reqs) or len(results) < len(reqs):
        now = time.perf_counter() - t_start
        while k < len(reqs) and reqs[k]["arrival"] <= now:
            r = reqs[k]
            ids[srv.submit(r["problem"], r["params"], r["steps"], lowmach=r["lowmach"])] = k
            k += 1
        for res in srv.poll():
            i = ids[res.id]
            results[i] = res
            if i in sample:
                keep[i] = srv.get_prim(res.id)
            srv.release(res.id)
        if k < len(reqs):
            time.sleep(max(0.0, min(0.002, reqs[k]["arrival"] - (time.perf_counter() - t_start))))
        else:
            time.sleep(0.0005)
    wall = time.perf_counter() - t_start
    st = srv.stats()
    cfgs = [config_name(st.bucket_cfg[b]) for b in range(4)]
    fam_cfgs = {"plain": config_name(st.bucket_cfg[0]), "diffusive": config_name(st.diff_cfg[0]),
                "extended": config_name(st.ext_cfg)}
    srv.close()
    tts = np.array([results[i].done_s - results[i].submit_s for i in range(len(reqs))])
    work = sum(float(r["N"]) ** 2 * results[i].steps for i, r in enumerate(reqs))
    first = min(results[i].submit_s for i in results)
    last = max(results[i].done_s for i in results)
    agg = work / (last - first)
    # plain FP64 path, one request at a time, on the sample
    sub = sorted(sample)
    s_work, s_time, err_rho, err_p, drift, service = 0.0, 0.0, [], [], [], []
    for i in sub:
        r = reqs[i]
        t0 = time.perf_counter()
        sim = fv.Simulation(r["params"], device=device)
        sim.init_problem(r["problem"])
        sim.advance(r["steps"], 1e30)
        q64 = sim.get_prim()
        el = time.perf_counter() - t0
        sim.close()
        service.append(el)
        s_work += float(r["N"]) ** 2 * r["steps"]
        s_time += el
        q32 = keep[i]
        err_rho.append(float(np.sum(np.abs(q32[..., 0] - q64[..., 0])) / np.sum(np.abs(q64[..., 0]))))
        err_p.append(float(np.sum(np.abs(q32[..., 3] - q64[..., 3])) / np.sum(np.abs(q64[..., 3]))))
        res = results[i]
        if r["kind"] != "sod":  # closed domains
            drift.append(abs(res.cons1[0] - res.cons0[0]) / abs(res.cons0[0]))
    plain_rate = s_work / s_time
    # FIFO single-server queueing of the sample through the plain path
    clock, tts64 = 0.0, []
    for i, sv in zip(sub, service):
        start = max(clock, reqs[i]["arrival"])
        clock = start + sv
        tts64.append(clock - reqs[i]["arrival"])
    return {
        "requests": len(reqs), "arrival_rate_hz": rate, "aggregate": agg, "unit": METRIC, "dtype": "f32 state/flux, "
        "f64 clock/dt/conservation sums/low-Mach energy recovery", "wall_s": wall, "cell_updates": work,
        "p50_s": float(np.percentile(tts, 50)), "p99_s": float(np.percentile(tts, 99)),
        "tile_configs_per_bucket": cfgs, "kernel_configurations": fam_cfgs, "replays": st.replays,
        "arena_reserved_gb": st.bytes_reserved / 1e9,
        "scheduling": ("shortest remaining work first, about %.3g cells per step" % active_cells) if active_cells > 0
        else "every admitted request at every step",
        "plain_fp64_one_at_a_time": {"sample": len(sub), "aggregate": plain_rate, "unit": METRIC,
                                     "p50_s": float(np.percentile(tts64, 50)),
                                     "p99_s": float(np.percentile(tts64, 99)),
                                     "note": "every 16th request, FIFO single server at the same arrival times"},
        "ratio_vs_plain_fp64": agg / plain_rate,
        "accuracy_vs_fp64": {"l1_rho_max": max(err_rho), "l1_rho_median": float(np.median(err_rho)),
                             "l1_p_max": max(err_p), "mass_drift_max": max(drift) if drift else None,
                             "sample": len(sub)},
    }


CHECKPOINTS = 8  # points of each error-versus-step curve


def checkpoints(steps, n=CHECKPOINTS):
    """Step counts at which an error curve is sampled: n points up to steps."""
    return sorted({max(1, round(steps * k / n)) for k in range(1, n + 1)})


def served_accuracy(fv, sample_every=16, device=0):
    """Accuracy of the batched FP32 service on the stream sample (every 16th
    request) against the plain FP64 path (bit-identical to the reference) run
    from the same initial condition, as error-versus-step curves: the service
    runs each request to every checkpoint (a request's result does not depend
    on what else is in the batch, so the runs to different step counts share
    one batch) and the FP64 path advances through the same checkpoints.  L1
    errors are sum |a - b| / sum |b| over the interior."""
    from fv2d_gb300.serve import Server, stream_requests, config_name
    reqs = stream_requests()
    sub = list(range(0, len(reqs), sample_every))
    pts = {i: checkpoints(reqs[i]["steps"]) for i in sub}
    q32 = {}
    res = {}
    # the kernel configurations the service runs in production (autotuned)
    with Server(budget_bytes=100e9, device=device, autotune=True) as srv:
        st = srv.stats()
        chosen = {"plain": config_name(st.bucket_cfg[0]), "diffusive": config_name(st.diff_cfg[0]),
                  "extended": config_name(st.ext_cfg)}
        ids = {}
        for i in sub:
            for n in pts[i]:
                ids[srv.submit(reqs[i]["problem"], reqs[i]["params"], n, lowmach=reqs[i]["lowmach"])] = (i, n)
        if srv.drain(1800) != 0:
            raise RuntimeError("the service did not finish the sample")
        for x in srv.poll():
            key = ids[x.id]
            res[key] = x
            q32[key] = srv.get_prim(x.id)
            srv.release(x.id)

    def l1(a, b, k):
        return float(np.sum(np.abs(a[..., k] - b[..., k])) / np.sum(np.abs(b[..., k])))

    rows = []
    for i in sub:
        r = reqs[i]
        sim = fv.Simulation(r["params"], device=device)
        sim.init_problem(r["problem"])
        curve, done = [], 0
        for n in pts[i]:
            sim.advance(n - done, 1e30)
            done = n
            q64 = sim.get_prim()
            x = res[(i, n)]
            curve.append([n, l1(q32[(i, n)], q64, 0), l1(q32[(i, n)], q64, 3)])
        sim.close()
        last = res[(i, pts[i][-1])]
        row = {"i": i, "kind": r["kind"], "N": r["N"], "steps": r["steps"], "status": last.status,
               "l1_rho": curve[-1][1], "l1_p": curve[-1][2], "curve": curve}
        if r["kind"] != "sod":  # closed domains: binary64 sums of the binary32 state
            row["mass_drift"] = abs(last.cons1[0] - last.cons0[0]) / abs(last.cons0[0])
        rows.append(row)
    summary = {"served_accuracy": True, "sample": len(rows),
               "median_l1_rho": float(np.median([w["l1_rho"] for w in rows])),
               "median_l1_p": float(np.median([w["l1_p"] for w in rows])),
               "l1_rho_le_1e-5": sum(w["l1_rho"] <= 1e-5 for w in rows),
               "mass_drift_max": max(w.get("mass_drift", 0.0) for w in rows), "kernel_configurations": chosen}
    return rows, summary


def run_reference(args, rank):
    if rank != 0:
        return
    cdt, upd, kind, what, cores = cpu_reference_sim(NX)
    for _ in range(args.warmup):
        upd(cdt())
    t0 = time.perf_counter()
    for _ in range(args.steps):
        upd(cdt())
    el = time.perf_counter() - t0
    v = NX * NY * args.steps / el
    line = {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (Sedov initial condition)",
            "config": config(NX, args.steps), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": cores, "kind": kind,
                             "sample": f"sedov {NX}x{NY}, {args.steps} iterations after {args.warmup} warm-up; "
                                       f"{what}"},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def fp32_configs(fv, reduced=False):
    """The two FP32-versus-FP64 benchmark set-ups, each to its end time:
    Kelvin-Helmholtz 4096^2 (CFL 0.7, t = 1) and Rayleigh-Taylor 1024 x 3072
    with gravity, conduction and viscosity (HLL, t = 5).  reduced=True: the
    same set-ups on a quarter of the cells per axis over the first eighth of
    their end times (KH 1024^2 to t = 0.125, RT 256 x 768 to t = 0.625), small
    enough for the CPU storage-floor runs of tests/accuracy_floor.py."""
    f = fv.as_float32
    d = 4 if reduced else 1
    e = 8.0 if reduced else 1.0
    return {
        "kh_%d_fp32_vs_fp64" % (4096 // d): ("kh_step", 1.0 / e, fv.default_params(
            Nx=4096 // d, Ny=4096 // d, gamma0=f(1.4), CFL=f(0.7), reconstruction=fv.PLM, riemann_solver=fv.HLLC,
            boundary_x=fv.BC_PERIODIC, boundary_y=fv.BC_PERIODIC, time_stepping=fv.TS_EULER)),
        "rt_%dx%d_fp32_vs_fp64" % (1024 // d, 3072 // d): ("rt_hydrostatic", 5.0 / e, fv.default_params(
            Nx=1024 // d, Ny=3072 // d, xmax=0.5, ymax=1.5, gamma0=f(1.4), CFL=f(0.8), reconstruction=fv.PLM,
            riemann_solver=fv.HLL, boundary_x=fv.BC_PERIODIC, boundary_y=fv.BC_REFLECTING,
            time_stepping=fv.TS_EULER, gravity_mode=fv.GRAV_CONSTANT, gy=f(-0.1),
            thermal_conductivity_active=1, kappa=f(1e-4), viscosity_active=1, mu=f(1e-4))),
    }


def fp32_vs_fp64(fv, problem, tend, p, device, stream, curve=False):
    """One set-up run to its end time by the plain FP64 path and by the served
    FP32 form from the same initial condition: L1 relative errors of rho and
    p at the end, conservation drift of mass, momentum and energy in both,
    and the rate of each whole run.  curve=True also gives the L1 errors at
    t = tend k / 8 (the FP64 run stops at each of those times on its way;
    the service runs the same request to each of them, after the timed
    run)."""
    import torch
    from fv2d_gb300.serve import Server
    cells = p.Nx * p.Ny
    area = (p.xmax - p.xmin) / p.Nx * (p.ymax - p.ymin) / p.Ny

    def sums(u):
        return [float(np.sum(u[..., k], dtype=np.float64)) * area for k in range(4)]

    def drift(c0, c1):
        # mass and energy relative to their start; momenta relative to the mass
        return {"mass": abs(c1[0] - c0[0]) / abs(c0[0]), "energy": abs(c1[3] - c0[3]) / abs(c0[3]),
                "momentum_x": abs(c1[1] - c0[1]) / abs(c0[0]), "momentum_y": abs(c1[2] - c0[2]) / abs(c0[0])}
    sim = fv.Simulation(p, device=device)
    sim.set_stream(stream.cuda_stream)
    sim.init_problem(problem)
    c0 = sums(sim.get_cons())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    marks = [tend * k / 8 for k in range(1, 8)] if curve else []
    at64 = {}
    s64, n64 = 0.0, 0
    for tk in marks + [tend]:
        e0.record(stream)
        t64, n, status = sim.advance(2 ** 31 - 1, tk)
        e1.record(stream)
        e1.synchronize()
        s64 += e0.elapsed_time(e1) * 1e-3
        n64 += n
        if tk != tend:
            at64[tk] = (t64, n64, sim.get_prim())
    q64 = sim.get_prim()
    c1 = sums(sim.get_cons())
    sim.close()
    with Server(budget_bytes=40e9, device=device, autotune=True) as srv:
        rid = srv.submit(problem, p, 2 ** 31 - 1, tend=tend)
        if srv.drain(3600) != 0:
            raise RuntimeError("the service did not finish " + problem)
        res = {r.id: r for r in srv.poll()}[rid]
        q32 = srv.get_prim(rid)
        srv.release(rid)
        ids = {srv.submit(problem, p, 2 ** 31 - 1, tend=tk): tk for tk in marks}
        if ids and srv.drain(3600) != 0:
            raise RuntimeError("the service did not finish " + problem)
        at32 = {}
        for r in srv.poll():
            at32[ids[r.id]] = (r.t, r.steps, srv.get_prim(r.id))
            srv.release(r.id)
    s32 = res.done_s - res.admit_s

    def l1(a, b, k):
        return float(np.sum(np.abs(a[..., k] - b[..., k])) / np.sum(np.abs(b[..., k])))
    points = [{"t_fp64": at64[tk][0], "t_fp32": at32[tk][0], "steps_fp64": at64[tk][1], "steps_fp32": at32[tk][1],
               "l1_rho": l1(at32[tk][2], at64[tk][2], 0), "l1_p": l1(at32[tk][2], at64[tk][2], 3)} for tk in marks]
    return {"problem": problem, "grid": [p.Nx, p.Ny], "tend": tend,
            "fp64": {"t": t64, "steps": n64, "seconds": s64, "rate": cells * n64 / s64, "unit": METRIC,
                     "drift": drift(c0, c1), "status": status},
            "fp32": {"t": res.t, "steps": res.steps, "seconds": s32, "rate": cells * res.steps / s32, "unit": METRIC,
                     "drift": drift(list(res.cons0), list(res.cons1)), "status": res.status,
                     "timing": "service clock, admission to completion (initial condition, steps, final sums)"},
            "l1_rho": l1(q32, q64, 0), "l1_p": l1(q32, q64, 3), "curve": points,
            "note": "both runs stop at the first t >= tend; their final times differ by less than one dt"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-4096", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--no-fp32-configs", action="store_true",
                    help="skip the FP32-vs-FP64 runs of the Kelvin-Helmholtz 4096^2 and Rayleigh-Taylor 1024x3072 "
                         "set-ups to their end times")
    ap.add_argument("--fp32-configs-only", action="store_true", help="only those two runs")
    ap.add_argument("--fp32-configs-reduced", action="store_true",
                    help="with --fp32-configs-only: the reduced set-ups (a quarter of the cells per axis, an eighth of "
                         "the end time)")
    ap.add_argument("--served-requests", type=int, default=512)
    ap.add_argument("--served-only", action="store_true", help="only the batched FP32 service on the stream")
    ap.add_argument("--served-profile", action="store_true",
                    help="fixed batch for kernel profiling: 12 Sedov 768^2 requests x 60 steps")
    ap.add_argument("--served-profile-steps", type=int, default=60,
                    help="--served-profile: steps per request (profile a launch well after the first replays, "
                         "when every request of the batch is resident)")
    ap.add_argument("--served-saturated", action="store_true",
                    help="service rate without arrival gaps: the request stream submitted at once")
    ap.add_argument("--served-accuracy", action="store_true",
                    help="per-request accuracy of the service on the stream sample against the FP64 path")
    ap.add_argument("--served-active-cells", type=float, default=8e6,
                    help="service scheduling: shortest remaining work first with about this many cells per step "
                         "(0: every admitted request advances at every step)")
    ap.add_argument("--served-single-launch", action="store_true",
                    help="--served-saturated / --served-only: every request in one work list and one launch per "
                         "step instead of one per grid-size bucket")
    ap.add_argument("--served-band", type=int, default=0,
                    help="--served-saturated / --served-profile: rows per work item of the march kernels (0: chosen "
                         "per lane)")
    ap.add_argument("--served-tile", default=None,
                    help="kernel configuration for every bucket of the profiling batch (e.g. 28/32x20/march)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        return run_reference(args, rank)

    import torch
    import fv2d_gb300 as fv
    if not os.path.exists(fv.LIB_PATH):
        from fv2d_gb300 import build as b
        b.build()
    if args.served_saturated:
        from fv2d_gb300.serve import Server, stream_requests, config_name
        reqs = stream_requests(n=args.served_requests)
        with Server(budget_bytes=150e9, device=local, autotune=args.served_tile is None,
                    tile_config=args.served_tile, active_cells=args.served_active_cells, band_rows=args.served_band,
                    single_launch=args.served_single_launch) as srv:
            t0 = time.perf_counter()
            for r in reqs:
                srv.submit(r["problem"], r["params"], r["steps"], lowmach=r["lowmach"])
            lat = []
            while len(lat) < len(reqs):
                for x in srv.poll():
                    lat.append(x.done_s - x.submit_s)
                    srv.release(x.id)
                time.sleep(0.0005)
            wall = time.perf_counter() - t0
            st = srv.stats()
            work = sum(float(r["N"]) ** 2 * r["steps"] for r in reqs)
            print(json.dumps({"served_saturated": True, "requests": len(reqs), "cell_updates": work,
                              "wall_s": wall, "rate": work / wall, "unit": METRIC,
                              "p50_s": float(np.median(lat)), "p99_s": float(np.percentile(lat, 99)),
                              "active_cells": args.served_active_cells, "single_launch": args.served_single_launch,
                              "tile_configs_per_bucket": [config_name(st.bucket_cfg[b]) for b in range(4)]}),
                  flush=True)
        return
    if args.served_accuracy:
        rows, summary = served_accuracy(fv, device=local)
        for w in rows:
            print(json.dumps(w), flush=True)
        print(json.dumps(summary), flush=True)
        return
    if args.fp32_configs_only:
        torch.cuda.set_device(local)
        stream = torch.cuda.Stream()
        for name, (problem, tend, pc) in fp32_configs(fv, args.fp32_configs_reduced).items():
            print(json.dumps({name: fp32_vs_fp64(fv, problem, tend, pc, local, stream, curve=True)}), flush=True)
        return
    if args.served_profile:
        from fv2d_gb300.serve import Server
        with Server(budget_bytes=20e9, device=local, autotune=False, tile_config=args.served_tile,
                    band_rows=args.served_band) as srv:
            p = workload_params(fv, 768)
            for _ in range(12):
                srv.submit("sedov", p, args.served_profile_steps)
            srv.drain(300)
            st = srv.stats()
            print(json.dumps({"served_profile": True, "completed": st.completed, "cell_updates": st.cell_updates,
                              "busy_s": st.busy_s}), flush=True)
        return
    if args.served_only:
        t0 = time.perf_counter()
        served = run_served(fv, n_requests=args.served_requests, device=local,
                            active_cells=args.served_active_cells, single_launch=args.served_single_launch)
        print(json.dumps({"metric": METRIC, "served": served, "wall_s": time.perf_counter() - t0,
                          "single_launch": args.served_single_launch}), flush=True)
        return
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    p = workload_params(fv, NX)
    sim = fv.Simulation(p, device=local)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)

    # warm-up on a first run, then restart from the initial condition so that
    # the timed region is iterations 0..K-1 of the Sedov problem
    sim.init_problem("sedov")
    sim.run_async(args.warmup)
    stream.synchronize()
    sim.init_problem("sedov")
    sim.set_time(0.0, 0)
    stream.synchronize()

    gpu_index = local
    cvd = os.environ.get("CUDA_VISIBLE_DEVICES")
    if cvd:
        ids = cvd.split(",")
        if local < len(ids) and ids[local].strip().isdigit():
            gpu_index = int(ids[local])
    sampler = ClockSampler(gpu_index)
    time.sleep(0.3)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(stream)
    sim.run_async(args.steps)
    e1.record(stream)
    e1.synchronize()
    barrier()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1)
    t_sim, ite = sim.time()
    if ite != args.steps:
        raise RuntimeError(f"expected {args.steps} iterations, device reports {ite}")
    ms_max = max_over_ranks(ms, dist, "cuda")
    cells = NX * NY
    value = whole_job_rate(cells * args.steps, world, ms_max * 1e-3)
    ms_step = ms_max / args.steps

    # roofline of the fused step kernel (one step launch + a one-thread commit per iteration)
    peak, peak_kind = measured_peaks()
    achieved = BYTES_PER_CELL * cells / (ms_step * 1e-3) / 1e9
    prof = profile_figures()
    traffic = prof.get("dram_bytes_per_cell")
    fp64_peak = fv.probe_fp64_peak(local)
    # The binding unit: binary64 pipe instructions (one per DFMA/DADD/DMUL/...),
    # peak = measured DFMA rate / 2 flops.
    pipe_peak = fp64_peak / 2.0
    fp64 = {"bound": "fp64_pipe", "peak": pipe_peak, "unit": "G fp64-pipe ops/s",
            "peak_kind": "measured DFMA loop (1255 GFLOP/s class) / 2", "achieved": None, "frac": None}
    if "fp64_pipe_ops_per_cell" in prof:
        ach = prof["fp64_pipe_ops_per_cell"] * cells / (ms_step * 1e-3) / 1e9
        fp64.update(achieved=ach, frac=ach / pipe_peak, ops_per_cell=prof["fp64_pipe_ops_per_cell"],
                    ops_source="ncu capture, profiles/step_fp64_plm_hllc_sedov.txt")

    # end to end through the C-ABI with host buffers
    q0 = torch.empty((NY, NX, 4), dtype=torch.float64, pin_memory=True)
    q1 = torch.empty_like(q0).pin_memory()
    sim.init_problem("sedov")
    sim.get_prim_ptr(q0.data_ptr())
    # q1 is the context's host mirror: each fv2d_update writes the new state into
    # it from the step kernel (over the host link, overlapped with the step)
    sim.set_host_mirror(q1.data_ptr())
    ke = max(1, args.e2e_steps)

    def e2e_steps(k):
        # per step: its input from page-locked host memory (the first by
        # set_prim, the others prefetched over the host link while the
        # previous step computes), dt, the step writing the host mirror, the
        # result read back
        sim.set_prim_ptr(q0.data_ptr())
        for n in range(k):
            sim.update(sim.compute_dt()[0])
            if n + 1 < k:
                sim.prefetch_prim_ptr(q0.data_ptr())
            sim.get_prim_ptr(q1.data_ptr())
            if n + 1 < k:
                sim.set_prim_ptr(q0.data_ptr())
    e2e_steps(2)
    barrier()
    t0 = time.perf_counter()
    e2e_steps(ke)
    el = time.perf_counter() - t0
    el_max = max_over_ranks(el, dist, "cuda")
    e2e = {"value": whole_job_rate(cells * ke, world, el_max), "unit": METRIC, "h2d_bytes_per_step": cells * 32,
           "d2h_bytes_per_step": cells * 32 + 8, "steps": ke,
           "path": "per step: its input from pinned host memory (fv2d_prefetch_prim during the previous step, "
                   "then fv2d_set_prim from the staged copy; the first step's set_prim reads the host link) + "
                   "fv2d_compute_dt + fv2d_update (writes the pinned host mirror while it computes) + "
                   "fv2d_get_prim(mirror: waits for the step)"}
    sim.set_host_mirror(0)

    extra = {}
    if not args.no_4096 and world == 1:
        p4 = workload_params(fv, 4096)
        s4 = fv.Simulation(p4, device=local)
        s4.set_stream(stream.cuda_stream)
        s4.init_problem("sedov")
        s4.run_async(5)
        stream.synchronize()
        k4 = max(10, args.steps // 10)
        e0.record(stream)
        s4.run_async(k4)
        e1.record(stream)
        e1.synchronize()
        ms4 = e0.elapsed_time(e1) / k4
        a4 = BYTES_PER_CELL * 4096 * 4096 / (ms4 * 1e-3) / 1e9
        extra["sedov_4096"] = {"value": 4096 * 4096 / (ms4 * 1e-3), "unit": METRIC, "steps": k4,
                               "ms_per_step": ms4, "hbm_achieved_gbs": a4, "hbm_frac": a4 / peak}
        s4.close()
        # the other two benchmark set-ups of the reference's scope (same binary64 path)
        f = fv.as_float32
        others = {
            "kh_4096": ("kh_step", fv.default_params(
                Nx=4096, Ny=4096, gamma0=f(1.4), CFL=f(0.7), reconstruction=fv.PLM, riemann_solver=fv.HLLC,
                boundary_x=fv.BC_PERIODIC, boundary_y=fv.BC_PERIODIC, time_stepping=fv.TS_EULER)),
            "rt_1024x3072": ("rt_hydrostatic", fv.default_params(
                Nx=1024, Ny=3072, xmax=0.5, ymax=1.5, gamma0=f(1.4), CFL=f(0.8), reconstruction=fv.PLM,
                riemann_solver=fv.HLL, boundary_x=fv.BC_PERIODIC, boundary_y=fv.BC_REFLECTING,
                time_stepping=fv.TS_EULER, gravity_mode=fv.GRAV_CONSTANT, gy=f(-0.1),
                thermal_conductivity_active=1, kappa=f(1e-4), viscosity_active=1, mu=f(1e-4))),
        }
        for name, (problem, po) in others.items():
            so = fv.Simulation(po, device=local)
            so.set_stream(stream.cuda_stream)
            so.init_problem(problem)
            so.run_async(5)
            stream.synchronize()
            ko = max(10, args.steps // 10)
            e0.record(stream)
            so.run_async(ko)
            e1.record(stream)
            e1.synchronize()
            mso = e0.elapsed_time(e1) / ko
            cells_o = po.Nx * po.Ny
            extra[name] = {"value": cells_o / (mso * 1e-3), "unit": METRIC, "steps": ko, "ms_per_step": mso,
                           "problem": problem, "grid": [po.Nx, po.Ny]}
            so.close()

    if world == 1 and not args.no_fp32_configs:
        for name, (problem, tend, pc) in fp32_configs(fv).items():
            extra[name] = fp32_vs_fp64(fv, problem, tend, pc, local, stream)

    served = None
    if world == 1 and not args.no_served:
        import numpy  # noqa: F401
        served = run_served(fv, n_requests=args.served_requests, device=local,
                            active_cells=args.served_active_cells)

    if rank != 0:
        return
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = cpu_oracle_rate(NX)
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (Sedov initial condition, seeded inputs)",
        "config": config(NX, args.steps),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": (traffic * cells) if traffic else None, "peak_kind": peak_kind,
                     "bytes_per_cell": BYTES_PER_CELL, "kernel": "fv2d::step_kernel<PLM,HLLC>",
                     "duration": "CUDA events per iteration: the step kernel plus its one-thread commit kernel "
                                 "(~4.7 us, 0.4 % of the iteration in the ncu launch list)",
                     "binding": "instruction issue, not HBM: binary64 pipe ~64 %, integer ALU ~55 % busy "
                                "(profiles/step_fp64_plm_hllc_sedov.txt); see roofline_fp64"},
        "roofline_fp64": fp64,
        "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
        "gpu_launches": 2 * args.steps + 1,  # begin_kernel, then step_kernel + commit_kernel per iteration
        "sim_time": t_sim,
        "served": served,
    }
    line.update(extra)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
