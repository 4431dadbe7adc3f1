#!/usr/bin/env python
"""Forward + adjoint WCSPH throughput on one GB300.

Workload ("single large instance"): a 1024 x 1024 jittered lattice (1,048,576
particles, dx = 1e-3, uniform jitter +-0.05 dx, seed 1) at the left of a
2.048 x 1.28 tank; h = 1.3 dx, rho0 = 1000, m = rho0 dx^2, c0 = 10 sqrt(2 g H),
mu = 0.02, kw = 5e4, dt = 0.25 h / c0; theta 256 x 256, seeded uniform [0,1]
smoothed by a 5 x 5 box filter (seed 2); 1000 steps in FP32 with a binomial
checkpoint tape of 32 snapshots; objective = kinetic energy of the right half.
A bench step is one complete solve (forward sweep, objective, reverse sweep
with recomputation). Metric: forward+adjoint particle-steps/s
(N x time steps / solve time). Synthetic data; no dataset is involved.

value: device-resident inputs (the initial state is cloned on the device),
timed with CUDA events on the library stream. e2e: the same solve through
the C ABI with host buffers (State from host X0, Array(X_T), host objective,
host seeds, Array(gradients)), wall-clock with the copies inside.
--impl reference: the CPU restatement of the reference (the Julia reference
cannot run here) on all host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# steps of the short solves that choose the block sizes inside the solve
TUNE_STEPS = 32

# ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch at 1,048,576
# particles, FP32 (the --set full captures summarised in profiles/*_1M_fp32.md)
TRAFFIC_1M_F32 = {
    "density": 38.243584e6 + 0.870144e6,
    "accel_integrate": 55.135488e6 + 2.096640e6,
    "accel_drag": 71.912192e6 + 3.559680e6,
    "pass1": 76.111104e6 + 3.872512e6,
    "pass2": 63.416832e6 + 0.484096e6,
}

# smsp__issue_active.avg.pct_of_peak_sustained_active of the same captures:
# the fraction of cycles in which a warp scheduler issued, the bound these
# gather kernels actually meet (HBM throughput stays in single digits)
ISSUE_ACTIVE_1M_F32 = {
    "density": 0.7623, "accel_integrate": 0.6856, "accel_drag": 0.6692,
    "pass1": 0.7149, "pass2": 0.7357,
}

# lts__throughput.avg.pct_of_peak_sustained_elapsed and
# l1tex__throughput.avg.pct_of_peak_sustained_active of the same captures:
# neither cache level is near its peak either
L2_L1_FRAC_1M_F32 = {
    "density": (0.0803, 0.3387), "accel_integrate": (0.0900, 0.6129),
    "accel_drag": (0.0929, 0.5730), "pass1": (0.0983, 0.6216), "pass2": (0.1094, 0.4152),
}

# algorithmic HBM bytes per particle per launch (compulsory traffic of the
# minimal dataflow, s = sizeof(T)): read/write sets of each fused pass
ALGO_WORDS = {
    "density": 4,          # read X (2) -> write p/rho^2, 1/rho (2)
    "accel_integrate": 10, # read X, V, pterm, invrho (6) -> write X', V' (4)
    "accel_drag": 15,      # read X, V, pterm, invrho, gX, gV (10) -> abar, galpha, gV (5)
    "pass1": 16,           # read abar, X, V, pterm, invrho, galpha, gV (11) -> gV, gXs, grho (5)
    "pass2": 9,            # read grho, X, gXs, gX (7) -> gX (2)
}


def workload(n_side=1024, nsteps=1000, snapshots=32, ntheta=256, dtype="f32"):
    dx = 1e-3
    H = n_side * dx
    h = 1.3 * dx
    c0 = 10.0 * math.sqrt(2 * 9.81 * H)
    p = dict(h=h, m=1000.0 * dx * dx, rho0=1000.0, c=c0, mu=0.02, dt=0.25 * h / c0,
             Lx=2.0 * H, Ly=1.25 * H, kw=5e4, ngx=ntheta, ngy=ntheta)
    rng = np.random.default_rng(1)
    xs = dx + dx * np.arange(n_side)
    X, Y = np.meshgrid(xs, xs)
    X0 = np.vstack([X.ravel(), Y.ravel()]) + rng.uniform(-0.05 * dx, 0.05 * dx, (2, n_side ** 2))
    V0 = np.zeros_like(X0)
    t = np.random.default_rng(2).random((ntheta, ntheta))
    pad = np.pad(t, 2, mode="edge")
    theta = sum(pad[i:i + ntheta, j:j + ntheta] for i in range(5) for j in range(5)) / 25.0
    cfg = {"workload": f"single large instance: {n_side}x{n_side} jittered lattice "
                       f"({n_side * n_side} particles), {nsteps} steps {dtype.upper()}, "
                       f"binomial checkpointing with {snapshots} snapshots, theta {ntheta}x{ntheta}",
           "particles": n_side * n_side, "time_steps": nsteps, "snapshots": snapshots,
           "theta": [ntheta, ntheta], "tank": [p["Lx"], p["Ly"]], "dx": dx,
           "skin": 0.2, "interval": 4, "maxnb": 64, "objective": "kinetic energy, right half",
           "l2": "inputs larger than L2 (checkpoint set and per-step arrays stream >1 GB per solve)"}
    return p, X0, V0, theta, cfg


def small_workload():
    """The reference's CPU-runnable dam break: a 56 x 37 block (2072 particles),
    dx = 0.01, origin (dx, dx), 1.6 x 1.0 tank, h = 1.3 dx, rho0 = 1000,
    c0 = 10 sqrt(2 g H), mu = 0.02, kw = 5e4, dt = 0.25 h / c0, theta 32 x 32 of
    zeros, 5333 steps in FP64 with a full tape."""
    dx, nx, ny = 0.01, 56, 37
    H = ny * dx
    h = 1.3 * dx
    c0 = 10.0 * math.sqrt(2 * 9.81 * H)
    p = dict(h=h, m=1000.0 * dx * dx, rho0=1000.0, c=c0, mu=0.02, dt=0.25 * h / c0, Lx=1.6,
             Ly=1.0, kw=5e4, ngx=32, ngy=32)
    xs = dx + dx * np.arange(nx)
    ys = dx + dx * np.arange(ny)
    X, Y = np.meshgrid(xs, ys)
    X0 = np.vstack([X.ravel(), Y.ravel()])
    cfg = {"workload": "small dam break: 56x37 = 2072 particles, 5333 steps FP64, full tape, "
                       "theta 32x32 zeros", "particles": nx * ny, "time_steps": 5333,
           "snapshots": 0, "theta": [32, 32], "tank": [1.6, 1.0], "dx": dx, "skin": 0.2,
           "interval": 4, "maxnb": 64, "objective": "kinetic energy, right half",
           "l2": "working set fits in L2 (2072 particles, ~1 MB per state); one timed step "
                 "is a whole 5333-step solve whose tape (0.35 GB) streams through HBM"}
    return p, X0, np.zeros_like(X0), np.zeros((32, 32)), cfg


def dense_workload(side=2896, ntheta=512, seed=5):
    """Dense stress case: a side x side block (8,386,816 particles for 2896)
    compressed 1.15x (spacing dx/1.15 with the mass of the uncompressed
    lattice), rebuilt every step, 200 steps, 16 checkpoints, theta 512 x 512
    with 50% solid cells in seeded random blobs (alpha 1000 vs 0)."""
    dx = 1e-3
    sp = dx / 1.15
    H = side * sp
    h = 1.3 * dx
    c0 = 10.0 * math.sqrt(2 * 9.81 * H)
    p = dict(h=h, m=1000.0 * dx * dx, rho0=1000.0, c=c0, mu=0.02, dt=0.25 * h / c0,
             Lx=2.0 * H, Ly=1.25 * H, kw=5e4, ngx=ntheta, ngy=ntheta)
    rng = np.random.default_rng(seed)
    xs = sp + sp * np.arange(side)
    X, Y = np.meshgrid(xs, xs)
    X0 = np.vstack([X.ravel(), Y.ravel()]) + rng.uniform(-0.05 * sp, 0.05 * sp, (2, side * side))
    f = rng.standard_normal((ntheta, ntheta))
    for _ in range(6):  # blobs: repeated 5x5 box smoothing
        pad = np.pad(f, 2, mode="wrap")
        f = sum(pad[i:i + ntheta, j:j + ntheta] for i in range(5) for j in range(5)) / 25.0
    theta = np.where(f > np.median(f), 1000.0, 0.0)
    cfg = {"workload": f"dense stress: {side}x{side} = {side * side} particles compressed 1.15x, "
                       "rebuilt every step, 200 steps FP32, 16 checkpoints, theta 512x512 "
                       "with 50% solid blobs", "particles": side * side, "time_steps": 200,
           "snapshots": 16, "theta": [ntheta, ntheta], "dx": sp, "skin": 0.2, "interval": 1,
           "maxnb": 64, "objective": "kinetic energy, right half",
           "l2": "inputs larger than L2 (8.4M particles: ~0.5 GB of per-particle arrays per pass)"}
    return p, X0, np.zeros_like(X0), theta, cfg


def batched_workload(B=64, nsteps=2000, ntheta=64, seed=3, snapshots=0):
    """64 independent dam breaks: N log-uniform in [1k, 64k], aspect (height /
    width of the water block) uniform in [0.3, 1.0], each with its own seeded,
    box-smoothed 64 x 64 theta; dx = 1e-3, tank 2W x 1.25 max(W, H)."""
    rng = np.random.default_rng(seed)
    dx = 1e-3
    inst = []
    for b in range(B):
        n = int(round(math.exp(rng.uniform(math.log(1000), math.log(64000)))))
        aspect = rng.uniform(0.3, 1.0)
        nx = max(2, int(round(math.sqrt(n / aspect))))
        ny = max(2, int(round(n / nx)))
        W, H = nx * dx, ny * dx
        h = 1.3 * dx
        c0 = 10.0 * math.sqrt(2 * 9.81 * H)
        p = dict(h=h, m=1000.0 * dx * dx, rho0=1000.0, c=c0, mu=0.02, dt=0.25 * h / c0,
                 Lx=2.0 * W, Ly=1.25 * max(W, H), kw=5e4, ngx=ntheta, ngy=ntheta)
        xs = dx + dx * np.arange(nx)
        ys = dx + dx * np.arange(ny)
        X, Y = np.meshgrid(xs, ys)
        X0 = np.vstack([X.ravel(), Y.ravel()]) + rng.uniform(-0.05 * dx, 0.05 * dx, (2, nx * ny))
        t = rng.random((ntheta, ntheta))
        pad = np.pad(t, 2, mode="edge")
        theta = sum(pad[i:i + ntheta, j:j + ntheta] for i in range(5) for j in range(5)) / 25.0
        inst.append((p, X0, np.zeros_like(X0), theta))
    cfg = {"workload": f"batched: {B} dam breaks, N log-uniform in [1k, 64k], aspect in [0.3, 1], "
                       f"own {ntheta}x{ntheta} theta each, {nsteps} steps FP32, "
                       + ("full tape" if snapshots == 0 else f"{snapshots} checkpoint slots"),
           "instances": B, "particles": int(sum(x[1].shape[1] for x in inst)),
           "time_steps": nsteps, "snapshots": snapshots, "theta": [ntheta, ntheta], "dx": dx,
           "skin": 0.2, "interval": 4, "maxnb": 64, "objective": "kinetic energy, right half",
           "l2": "inputs larger than L2 (per-particle arrays of all instances, and the "
                 "tape or checkpoints, stream through HBM every solve)"}
    return inst, cfg


def run_batched(args):
    """Packed batch (one launch per kernel for all instances) vs the same
    solves run one after another, one solve per launch sequence."""
    import torch
    import sphadjoint_gb300 as S
    from sphadjoint_gb300 import _lib as LB

    torch.cuda.set_device(0)
    L = S.load()
    stream = torch.cuda.Stream()
    LB.check(L.sph_set_stream(C.c_void_p(stream.cuda_stream)))
    inst, cfg = batched_workload(args.instances, args.nsteps, snapshots=args.snapshots)
    ps = [S.SPHParams(**p, dtype=args.dtype) for p, _, _, _ in inst]
    ntot = sum(x[1].shape[1] for x in inst)
    flags = C.c_uint32()

    bt0 = S.Batch([x[1] for x in inst], [x[2] for x in inst], ps)
    bt = S.Batch([x[1] for x in inst], [x[2] for x in inst], ps)
    th = S.BatchField([x[3] for x in inst], args.dtype)
    tape = S.Tape(ntot, args.nsteps, ps[0], snapshots=args.snapshots)
    ws = S.BatchWorkspace(bt)
    Jb = (C.c_double * len(inst))()

    def solve_batch(nsteps=None, tp=None):
        nsteps, tp = nsteps or args.nsteps, tp or tape
        LB.check(L.sph_state_assign(bt.h, bt0.h))
        tp.reset()
        LB.check(L.sph_simulate(bt.h, th.h, None, nsteps, tp.h, C.byref(flags)))
        LB.check(L.sph_batch_objective(ws.h, bt.h, 0, None, Jb))
        LB.check(L.sph_backward_seeded(ws.h, tp.h, th.h, None, None, 0.2, 4, 64, C.byref(flags)))

    if args.autotune:
        b6 = (C.c_int32 * 6)()
        LB.check(L.sph_autotune(bt.h, th.h, 5, b6))
        tape_t = S.Tape(ntot, TUNE_STEPS, ps[0], snapshots=0)
        solve_batch(TUNE_STEPS, tape_t)  # first use allocates
        S.autotune_in_solve(bt, lambda: solve_batch(TUNE_STEPS, tape_t))
        del tape_t

    def timed(fn, reps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = L.sph_launch_count()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, (L.sph_launch_count() - n0) / reps

    graph = None
    if args.graph:
        # the whole batched solve recorded once as a CUDA graph, replayed per step
        for _ in range(max(1, args.warmup)):
            solve_batch()
        torch.cuda.synchronize()
        graph = S.capture(solve_batch)
    ms_b, launches_b = timed(graph.launch if graph is not None else solve_batch, args.steps)
    graph = None
    del tape

    # the same instances, one solve at a time
    solo = []
    for p, X0, V0, theta in inst:
        pp = S.SPHParams(**p, dtype=args.dtype)
        n = X0.shape[1]
        s0 = S.State(X0, V0, pp)
        s1 = S.State(X0, V0, pp)
        f = S.DesignField(theta, args.dtype)
        tp = S.Tape(n, args.nsteps, pp, snapshots=args.snapshots)
        w = S.AdjointWorkspace(n, pp)
        solo.append((pp, s0, s1, f, tp, w))
    Js = C.c_double()

    def solve_plain():
        for pp, s0, s1, f, tp, w in solo:
            pc = pp.c_struct()
            LB.check(L.sph_state_assign(s1.h, s0.h))
            tp.reset()
            LB.check(L.sph_simulate(s1.h, f.h, C.byref(pc), args.nsteps, tp.h, C.byref(flags)))
            LB.check(L.sph_objective(w.h, s1.h, 0, None, C.byref(pc), C.byref(Js)))
            LB.check(L.sph_backward_seeded(w.h, tp.h, f.h, C.byref(pc), None, 0.2, 4, 64,
                                           C.byref(flags)))

    ms_p, launches_p = timed(solve_plain, max(1, args.steps // 2))
    ps_total = ntot * args.nsteps
    line = {"metric": "fwd+adjoint particle-steps/s (batched vs one solve per launch)",
            "value": ps_total / (ms_b / 1000.0), "unit": "particle-steps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_b,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": args.dtype, "data": "synthetic", "config": cfg,
            "plain": {"value": ps_total / (ms_p / 1000.0), "ms_per_step": ms_p,
                      "gpu_launches_per_step": launches_p},
            "speedup_vs_plain": ms_p / ms_b, "gpu_launches": launches_b,
            "graph": bool(args.graph)}
    print(json.dumps(line))


def served_requests(R, rate, seed=4, ntheta=128, n_range=(2000, 200000),
                    steps_range=(500, 5000), snapshots=32):
    """Requests of a topology-optimisation line search: N uniform in
    [2k, 200k] (square jittered lattice, dx = 1e-3), steps uniform in
    [500, 5000], theta = base 128 x 128 design + step * direction with the step
    log-uniform in [1e-3, 1e-1]; Poisson arrivals at `rate` per second."""
    rng = np.random.default_rng(seed)

    def smooth(a):
        pad = np.pad(a, 2, mode="edge")
        return sum(pad[i:i + ntheta, j:j + ntheta] for i in range(5) for j in range(5)) / 25.0

    base = smooth(rng.random((ntheta, ntheta)))
    direction = smooth(rng.standard_normal((ntheta, ntheta)))
    direction /= np.max(np.abs(direction))
    dx = 1e-3
    reqs, t = [], 0.0
    for _ in range(R):
        t += rng.exponential(1.0 / rate)
        n = int(rng.uniform(*n_range))
        side = max(2, int(round(math.sqrt(n))))
        steps = int(rng.uniform(*steps_range))
        step = math.exp(rng.uniform(math.log(1e-3), math.log(1e-1)))
        H = side * dx
        h = 1.3 * dx
        c0 = 10.0 * math.sqrt(2 * 9.81 * H)
        p = dict(h=h, m=1000.0 * dx * dx, rho0=1000.0, c=c0, mu=0.02, dt=0.25 * h / c0,
                 Lx=2.0 * H, Ly=1.25 * H, kw=5e4, ngx=ntheta, ngy=ntheta)
        xs = dx + dx * np.arange(side)
        X, Y = np.meshgrid(xs, xs)
        X0 = np.vstack([X.ravel(), Y.ravel()]) + rng.uniform(-0.05 * dx, 0.05 * dx,
                                                               (2, side * side))
        theta = np.clip(base + step * direction, 0.0, 1.0)
        reqs.append(dict(t=t, p=p, X0=X0, V0=np.zeros_like(X0), theta=theta, steps=steps,
                         snapshots=snapshots))
    return reqs


def served_sweep(args):
    """Poisson streams of forward + adjoint requests (the configuration's
    topology-optimisation line search) through the packed server, against the
    same requests served one at a time.

    served: the packed server (every request in flight advances one step per
    tick, each pass one launch over all of them), admitting requests FIFO by
    HBM bytes; each rate's stream replayed in real time, latency = submit to
    done. plain: the requests solved one at a time through the one-worker
    stream server (the solve-per-call path), submitted back to back so each
    service time is measured on the GPU; each rate's latencies are the FIFO
    replay of those service times against that rate's arrival times (one at a
    time, a request's solve does not depend on when it arrives). Both use the
    same tape per request: the full tape when it takes at most an eighth of
    the HBM budget, else the checkpoint snapshots that fit there."""
    import torch
    import sphadjoint_gb300 as S
    from sphadjoint_gb300.serve import Server

    S.load()
    rates = [float(r) for r in args.rates.split(",")]
    budget = int(args.hbm_budget_gb * (1 << 30))
    nr = tuple(int(x) for x in args.served_n.split(","))
    sr = tuple(int(x) for x in args.served_steps.split(","))

    def served_requests_cfg(R, rate):
        return served_requests(R, rate, n_range=nr, steps_range=sr)

    base = served_requests_cfg(args.requests, rates[0])
    P = [S.SPHParams(**q["p"], dtype=args.dtype) for q in base]
    snaps = [S.tape_plan(q["X0"].shape[1], q["steps"], p, budget // 8)[0]
             for q, p in zip(base, P)]
    ps_req = [q["X0"].shape[1] * q["steps"] for q in base]

    def warm(srv):
        w = served_requests(2, 1000.0, seed=99, n_range=(2000, 4000), steps_range=(50, 60))
        for q in w:
            srv.submit(S.SPHParams(**q["p"], dtype=args.dtype), q["X0"], q["V0"], q["theta"],
                       q["steps"], snapshots=0).wait()
        srv.reset_stats()
        srv.tickets.clear()

    def pct(a, f):
        a = sorted(a)
        k = f * (len(a) - 1)
        i = int(k)
        j = min(i + 1, len(a) - 1)
        return a[i] + (a[j] - a[i]) * (k - i)

    served = []
    for rate in rates:
        reqs = served_requests_cfg(args.requests, rate)
        with Server(hbm_budget_bytes=budget, dtype=args.dtype, packed=True,
                    max_inflight=args.max_inflight) as srv:
            warm(srv)
            t0 = time.perf_counter()
            tickets = []
            for q, p, c in zip(reqs, P, snaps):
                delay = q["t"] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                tickets.append(srv.submit(p, q["X0"], q["V0"], q["theta"], q["steps"],
                                          snapshots=c))
            for tk in tickets:
                tk.wait()
            st = srv.stats()
        served.append({"rate_per_s": rate, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                       "particle_steps_per_s": st["particle_steps_per_s"],
                       "completed": st["completed"], "peak_inflight": st["peak_inflight"],
                       "peak_admitted_gb": st["peak_bytes"] / (1 << 30)})

    # plain: the same requests one at a time, back to back
    with Server(workers=1, hbm_budget_bytes=budget, dtype=args.dtype) as srv:
        warm(srv)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        done = []
        tickets = [srv.submit(p, q["X0"], q["V0"], q["theta"], q["steps"], snapshots=c)
                   for q, p, c in zip(base, P, snaps)]
        for tk in tickets:
            tk.wait()
            done.append(time.perf_counter() - t0)
    service = [done[0]] + [done[k] - done[k - 1] for k in range(1, len(done))]
    plain = []
    for rate in rates:
        reqs = served_requests_cfg(args.requests, rate)
        free, lat = 0.0, []
        for q, sv in zip(reqs, service):
            start = max(q["t"], free)
            free = start + sv
            lat.append(1000.0 * (free - q["t"]))
        span = free - reqs[0]["t"]
        plain.append({"rate_per_s": rate, "p50_ms": pct(lat, 0.5), "p99_ms": pct(lat, 0.99),
                      "particle_steps_per_s": sum(ps_req) / span,
                      "completed": len(lat)})
    for a, b in zip(served, plain):
        a["vs_plain"] = a["particle_steps_per_s"] / b["particle_steps_per_s"]
    return {"workload": "served topology-optimisation line search: Poisson arrivals at each "
                        "rate, N uniform in [2k, 200k], steps uniform in [500, 5000], theta = "
                        "base 128x128 + log-uniform step along a fixed direction",
            "requests_per_rate": args.requests, "rates": rates,
            "hbm_budget_gb": args.hbm_budget_gb,
            "tape": "full tape when it takes at most 1/8 of the budget, else the snapshots "
                    "that fit there",
            "full_tape_requests": sum(1 for c in snaps if c == 0),
            "particle_steps_per_rate": sum(ps_req),
            "served": served, "plain": plain,
            "plain_method": "service times measured one at a time back to back; latencies are "
                            "their FIFO replay against each rate's arrival times",
            "plain_total_s": done[-1],
            "vs_plain_min": min(a["vs_plain"] for a in served)}


def run_served(args):
    """--workload served: the served sweep alone, as its own JSON line."""
    import torch

    torch.cuda.set_device(0)
    out = served_sweep(args)
    best = max(out["served"], key=lambda r: r["particle_steps_per_s"])
    line = {"metric": "served fwd+adjoint particle-steps/s and p50/p99 latency vs plain",
            "value": best["particle_steps_per_s"], "unit": "particle-steps/s", "n_gpus": 1,
            "higher_is_better": True, "dtype": args.dtype, "data": "synthetic",
            "config": {"workload": out["workload"]}, "served": out}
    print(json.dumps(line))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "power.draw", "clocks_event_reasons.active",
              "clocks_event_reasons.hw_slowdown", "clocks_event_reasons.hw_thermal_slowdown",
              "clocks_event_reasons.sw_thermal_slowdown", "clocks_event_reasons.sw_power_cap"]

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == len(self.FIELDS):
                self.rows.append(parts)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if not self.rows:
            return None
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if r[4 + k].lower() in ("active", "0x1", "1")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def replicas_value(ms_local, particle_steps_local):
    """Whole-job throughput of independent replicas (one solve stream per
    rank, no data-path collective): the slowest rank's time bounds the job,
    and every rank's work counts. Returns (ms_max, particle-steps/s)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(ms_local), float(particle_steps_local)], dtype=torch.float64)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
        ms = t[:1].to(dev)
        work = t[1:].to(dev)
        dist.all_reduce(ms, op=dist.ReduceOp.MAX)
        dist.all_reduce(work, op=dist.ReduceOp.SUM)
        t = torch.cat([ms.cpu(), work.cpu()])
    ms_max, work = float(t[0]), float(t[1])
    return ms_max, work / (ms_max / 1000.0)


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_sample(p, X0, V0, theta, dtype, budget_s=12.0, max_steps=64, interval=4):
    """Time the oracle (forward + adjoint with a full tape) on all host cores
    on the first few time steps of the workload; returns particle-steps/s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    o = O.Oracle(dtype)
    op = O.params(**p)
    th = o.theta(theta)
    N = X0.shape[1]

    def run(nsteps):
        st = o.state(op, X0, V0, interval=interval)
        tp = o.tape(N, nsteps)
        t0 = time.perf_counter()
        o.simulate(st, th, op, nsteps, tp)
        X, V = st.get()
        right = X[:, 0] > p["Lx"] / 2
        sV = np.where(right[:, None], p["m"] * V, 0.0)
        ws = o.workspace(N, op)
        o.backward(ws, tp, th, op, np.zeros_like(X), sV, interval=interval)
        return time.perf_counter() - t0

    t1 = run(1)
    n = int(max(1, min(max_steps, budget_s / max(t1, 1e-3))))
    t = run(n) if n > 1 else t1
    return {"value": N * n / t, "unit": "particle-steps/s", "cores": O.get_threads(),
            "kind": "port", "time_steps": n,
            "sample": f"{N} particles x {n} time steps, forward + adjoint with a full tape, "
                      f"{dtype.upper()}, C restatement of the reference with OpenMP",
            "seconds": t}


MODELS = {
    # the reference's physics: linear EOS, Morris viscosity (parity pinned)
    "reference": {},
    # the physics the benchmark configurations name (Tait EOS gamma = 7,
    # artificial viscosity alpha = 0.02); no counterpart in the reference
    "tait-av": dict(eos=1, gamma=7, visc=1, alpha=0.02),
}


def select_workload(args):
    """(params, X0, V0, theta, config, interval) of --workload and --model;
    small and dense fix their own steps, snapshots and precision."""
    interval = 4
    if args.workload == "small":
        p_d, X0, V0, theta, cfg = small_workload()
        args.dtype, args.nsteps, args.snapshots = "f64", 5333, 0
    elif args.workload == "dense":
        p_d, X0, V0, theta, cfg = dense_workload()
        args.nsteps, args.snapshots, interval = 200, 16, 1
    else:
        p_d, X0, V0, theta, cfg = workload(args.side, args.nsteps, args.snapshots, args.ntheta,
                                           args.dtype)
    p_d = dict(p_d, **MODELS[args.model])
    cfg = dict(cfg, model=args.model)
    if args.model != "reference":
        cfg["workload"] += ", Tait EOS (gamma 7) + artificial viscosity (alpha 0.02)"
    return p_d, X0, V0, theta, cfg, interval


def run_reference(args):
    ws, rank, _ = dist_info()
    p, X0, V0, theta, cfg, interval = select_workload(args)
    if rank != 0:
        return
    budget = args.ref_step_seconds
    for _ in range(args.warmup):
        cpu_sample(p, X0, V0, theta, args.dtype, budget_s=budget / 4, max_steps=2,
                   interval=interval)
    tot_ps, tot_t = 0.0, 0.0
    last = None
    for _ in range(args.steps):
        last = cpu_sample(p, X0, V0, theta, args.dtype, budget_s=budget,
                          max_steps=args.nsteps if args.workload == "small" else 64,
                          interval=interval)
        tot_ps += last["value"] * last["seconds"]
        tot_t += last["seconds"]
    v = tot_ps / tot_t
    line = {"impl": "reference", "metric": "fwd+adjoint particle-steps/s", "value": v,
            "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": args.dtype, "data": "synthetic", "config": cfg,
            "cpu_baseline": {k: last[k] for k in ("unit", "cores", "kind", "sample")} | {"value": v},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "horizon": {"sampled_time_steps": last["time_steps"], "sampled_tape": "full",
                        "configured_time_steps": args.nsteps,
                        "configured_snapshots": args.snapshots,
                        "note": "each step times the first sampled_time_steps steps of the "
                                "workload, forward + adjoint with a full tape (no checkpoint "
                                "recomputation), normalised per particle-step; the GPU arm runs "
                                "the configured horizon with checkpoint recomputation"},
            "note": "the reference is Julia (KernelAbstractions); Julia is not installed, so its "
                    "CPU path is timed through the C restatement in oracle/"}
    print(json.dumps(line))


def run_ours(args):
    import torch

    world, rank, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    import sphadjoint_gb300 as S
    from sphadjoint_gb300 import _lib as LB

    L = S.load()
    stream = torch.cuda.Stream()
    LB.check(L.sph_set_stream(C.c_void_p(stream.cuda_stream)))
    S.set_density_form(args.density_form)
    S.set_launch_overlap(bool(args.overlap))
    S.set_step_graphs(args.step_graphs)

    p_d, X0, V0, theta, cfg, interval = select_workload(args)
    p = S.SPHParams(**p_d, dtype=args.dtype)
    N = X0.shape[1]
    pc = p.c_struct()
    st0 = S.State(X0, V0, p, interval=interval)  # pristine initial state (device)
    st = S.State(X0, V0, p, interval=interval)
    th = S.DesignField(theta, args.dtype)
    tape = S.Tape(N, args.nsteps, p, snapshots=args.snapshots)
    ws = S.AdjointWorkspace(N, p)
    flags = C.c_uint32()
    J = C.c_double()

    def solve():
        LB.check(L.sph_state_assign(st.h, st0.h))
        tape.reset()
        LB.check(L.sph_simulate(st.h, th.h, C.byref(pc), args.nsteps, tape.h, C.byref(flags)))
        LB.check(L.sph_objective(ws.h, st.h, 0, None, C.byref(pc), C.byref(J)))
        LB.check(L.sph_backward_seeded(ws.h, tape.h, th.h, C.byref(pc), None, 0.2, interval, 64,
                                       C.byref(flags)))

    blocks = None
    if args.autotune:
        # block sizes: the engine's autotune on this workload's initial state,
        # then each kernel's fastest size inside short solves of the workload
        b6 = (C.c_int32 * 6)()
        LB.check(L.sph_autotune(st.h, th.h, 5, b6))
        tape_t = S.Tape(N, TUNE_STEPS, p, snapshots=0)

        def solve_short():
            LB.check(L.sph_state_assign(st.h, st0.h))
            tape_t.reset()
            LB.check(L.sph_simulate(st.h, th.h, C.byref(pc), TUNE_STEPS, tape_t.h,
                                    C.byref(flags)))
            LB.check(L.sph_objective(ws.h, st.h, 0, None, C.byref(pc), C.byref(J)))
            LB.check(L.sph_backward_seeded(ws.h, tape_t.h, th.h, C.byref(pc), None, 0.2,
                                           interval, 64, C.byref(flags)))

        solve_short()  # first use allocates
        blocks = dict(zip(S.TUNED_KERNELS, S.autotune_in_solve(st, solve_short)))
        del tape_t
    for _ in range(args.warmup):
        solve()
    torch.cuda.synchronize()
    graph = None
    if args.graph:
        # the whole solve recorded once as a CUDA graph and replayed per step
        graph = S.capture(solve)
        for _ in range(2):
            graph.launch()
        torch.cuda.synchronize()
        args.kernel_events = 0  # replays carry no per-launch events
    run_step = graph.launch if graph is not None else solve

    kid = LB.KERNEL_ID[args.kernel]
    LB.check(L.sph_profile_reset())
    LB.check(L.sph_profile_enable(kid, int(args.kernel_events)))
    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    clocks.start()
    torch.cuda.synchronize()
    n0 = L.sph_launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        run_step()
    e1.record(stream)
    torch.cuda.synchronize()
    launches = L.sph_launch_count() - n0
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    if graph is not None:
        LB.check(L.sph_workspace_objective_value(ws.h, C.byref(J)))
    kms, kn = C.c_double(), C.c_int64()
    LB.check(L.sph_profile_read(kid, C.byref(kms), C.byref(kn)))
    LB.check(L.sph_profile_enable(kid, 0))
    rec = tape.recomputed_steps()
    ms, value = replicas_value(ms, N * args.nsteps * args.steps)
    esz = 4 if args.dtype == "f32" else 8
    hbm, peak_kind = peaks()
    events_pass = None
    if not args.kernel_events:
        # the timed region ran without per-launch events; time the kernel in a
        # second pass of the same K solves, with events around each of its
        # launches (the solve itself runs launch by launch there)
        LB.check(L.sph_profile_reset())
        LB.check(L.sph_profile_enable(kid, 1))
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        f0.record(stream)
        for _ in range(args.steps):
            solve()
        f1.record(stream)
        torch.cuda.synchronize()
        LB.check(L.sph_profile_read(kid, C.byref(kms), C.byref(kn)))
        LB.check(L.sph_profile_enable(kid, 0))
        events_pass = {"solves": args.steps, "ms_per_step": f0.elapsed_time(f1) / args.steps}
    per_launch_ms = kms.value / max(kn.value, 1)
    algo_bytes = ALGO_WORDS[args.kernel] * esz * N
    achieved = algo_bytes / (per_launch_ms / 1000.0) / 1e9
    roof = {"kernel": args.kernel, "bound": "hbm", "achieved": achieved, "peak": hbm,
            "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": (args.traffic_bytes if args.traffic_bytes
                        else TRAFFIC_1M_F32.get(args.kernel)
                        if N == 1 << 20 and args.dtype == "f32" else None),
            "algorithmic_bytes_per_launch": algo_bytes, "ms_per_launch": per_launch_ms,
            "launches": kn.value,
            "issue_active_frac": (ISSUE_ACTIVE_1M_F32.get(args.kernel)
                                  if N == 1 << 20 and args.dtype == "f32" else None),
            "l2_l1_throughput_frac": (L2_L1_FRAC_1M_F32.get(args.kernel)
                                      if N == 1 << 20 and args.dtype == "f32" else None),
            "events": ("in the timed region" if args.kernel_events else
                       "second pass of the same K solves, events around each launch"),
            "events_pass": events_pass}

    # per-kernel breakdown of one more solve (untimed)
    kernels = {}
    if args.breakdown and rank == 0:
        for k in LB.KERNELS:
            L.sph_profile_enable(LB.KERNEL_ID[k], 1)
        L.sph_profile_reset()
        solve()
        torch.cuda.synchronize()
        for k in LB.KERNELS:
            a, b = C.c_double(), C.c_int64()
            L.sph_profile_read(LB.KERNEL_ID[k], C.byref(a), C.byref(b))
            if b.value:
                kernels[k] = {"ms": round(a.value, 3), "launches": b.value}
            L.sph_profile_enable(LB.KERNEL_ID[k], 0)

    # Whole-solve roofline: algorithmic HBM bytes of every executed pass (the
    # minimal dataflow's compulsory traffic, s = sizeof T): forward step 14s
    # (density 4s + accel/integrate 10s), reverse step 48s (tape read 4s,
    # density 4s, accel/drag 15s, pass 1 16s, pass 2 9s), the full tape's
    # write 4s per step, a neighbour rebuild 4s + 12; snapshot copies are not
    # counted. Rebuilds per solve are the build launches of the breakdown solve
    # when it ran, else one per `interval` executed steps.
    fwd_steps = args.nsteps + rec
    rebuilds = (kernels["nl_build"]["launches"] if "nl_build" in kernels
                else (fwd_steps + args.nsteps) // max(interval, 1))
    solve_bytes = N * (14 * esz * fwd_steps + 48 * esz * args.nsteps
                       + (4 * esz * args.nsteps if args.snapshots == 0 else 0)
                       + (4 * esz + 12) * rebuilds)
    solve_gbs = solve_bytes / (ms / args.steps / 1000.0) / 1e9  # per GPU
    solve_roof = {"bound": "hbm", "achieved": solve_gbs, "peak": hbm, "unit": "GB/s",
                  "frac": solve_gbs / hbm, "bytes_per_solve": solve_bytes,
                  "forward_steps": fwd_steps, "reverse_steps": args.nsteps,
                  "rebuilds": rebuilds}
    # the same per pass, from the breakdown solve's event-timed launches
    pass_roof = {}
    for k, words in ALGO_WORDS.items():
        if k in kernels and kernels[k]["ms"] > 0:
            gbs = words * esz * N * kernels[k]["launches"] / (kernels[k]["ms"] / 1000.0) / 1e9
            pass_roof[k] = {"achieved": round(gbs, 1), "frac": round(gbs / hbm, 4)}

    # the same solve in FP64 on the GPU (the FP64 oracle run of the workload):
    # relative difference of the FP32 results, max |a - b| / max |b|
    fp64 = None
    if args.fp64_check and args.dtype == "f32" and rank == 0:
        def grab(st_, ws_):
            X_, V_ = st_.get()
            gX_, gV_, gt_ = ws_.get()
            return {k: np.asarray(a, np.float64) for k, a in
                    (("X", X_), ("V", V_), ("gX", gX_), ("gV", gV_), ("gtheta", gt_))}

        solve()
        torch.cuda.synchronize()
        r32 = grab(st, ws)
        J32 = J.value
        p64 = S.SPHParams(**p_d, dtype="f64")
        st64 = S.State(X0, V0, p64, interval=interval)
        th64 = S.DesignField(theta, "f64")
        tp64 = S.Tape(N, args.nsteps, p64, snapshots=args.snapshots)
        ws64 = S.AdjointWorkspace(N, p64)
        t0 = time.perf_counter()
        S.simulate(st64, th64, p64, args.nsteps, tp64)
        J64 = ws64.objective(st64, "ke_right")
        S.backward_seeded(ws64, tp64, th64, p64, interval=interval)
        r64 = grab(st64, ws64)
        fp64 = {"seconds": time.perf_counter() - t0, "time_steps": args.nsteps,
                "objective": "kinetic energy, right half", "J_f32": J32, "J_f64": J64,
                "J_rel": abs(J32 - J64) / abs(J64)}
        for k in r64:
            fp64[k + "_rel"] = float(np.max(np.abs(r32[k] - r64[k])) /
                                     max(np.max(np.abs(r64[k])), 1e-300))
        del st64, tp64, ws64
        # The same comparison where the problem is still well conditioned: 10
        # steps of the smooth target objective centred in the block (the
        # right-half kinetic energy counts particles with x > Lx/2, and this
        # state's last lattice column sits on that line). IEEE FP32 itself
        # stays within 1e-5 of FP64 here on X, dJ/dX0, dJ/dV0 and J.
        H = N ** 0.5 * cfg["dx"]
        targs = (0.5 * H, 0.4 * H, 0.15 * H)
        short = {"time_steps": 10, "objective": "target_objective, centre (0.5H, 0.4H), "
                                                "sigma 0.15H"}
        res = {}
        for dt in ("f32", "f64"):
            pp = S.SPHParams(**p_d, dtype=dt)
            s_ = S.State(X0, V0, pp, interval=interval)
            t_ = S.Tape(N, 10, pp, snapshots=0)
            w_ = S.AdjointWorkspace(N, pp)
            S.simulate(s_, S.DesignField(theta, dt), pp, 10, t_)
            Jv = w_.objective(s_, "target", targs)
            S.backward_seeded(w_, t_, S.DesignField(theta, dt), pp, interval=interval)
            res[dt] = grab(s_, w_) | {"J": Jv}
            del s_, t_, w_
        for k in ("X", "V", "gX", "gV", "gtheta"):
            short[k + "_rel"] = float(np.max(np.abs(res["f32"][k] - res["f64"][k])) /
                                      max(np.max(np.abs(res["f64"][k])), 1e-300))
        short["J_rel"] = abs(res["f32"]["J"] - res["f64"]["J"]) / abs(res["f64"]["J"])
        fp64["well_conditioned"] = short

    # e2e: the reference-facing calls with host buffers
    e2e = None
    if args.e2e_steps > 0:
        # host buffers in pinned (page-locked) memory, as a caller that
        # streams solves would hold them; pageable numpy if pinning fails
        keep = []
        pinned_ok = [True]

        def host(shape, order="C"):
            try:
                t = torch.empty(int(np.prod(shape)), pin_memory=True,
                                dtype=torch.float64 if p.np == np.float64 else torch.float32)
                keep.append(t)
                return t.numpy().reshape(shape, order=order)
            except RuntimeError:
                pinned_ok[0] = False
                return np.empty(shape, p.np, order=order)

        Xh = host(X0.T.shape)
        Xh[...] = X0.T
        Vh = host(V0.T.shape)
        Vh[...] = V0.T
        thh = host(theta.shape, order="F")
        thh[...] = theta
        outX, outV, gX, gV = (host(Xh.shape) for _ in range(4))
        sV = host(Vh.shape)
        gth = host((p.ngx, p.ngy))

        def solve_host():
            h = C.c_void_p()
            LB.check(L.sph_state_create(C.byref(pc), N, Xh.ctypes.data_as(C.c_void_p),
                                        Vh.ctypes.data_as(C.c_void_p), p.code, 0.2, interval, 64,
                                        C.byref(h)))
            LB.check(L.sph_field_upload(th.h, thh.ctypes.data_as(C.c_void_p)))
            tape.reset()
            LB.check(L.sph_simulate(h, th.h, C.byref(pc), args.nsteps, tape.h, C.byref(flags)))
            LB.check(L.sph_state_get(h, outX.ctypes.data_as(C.c_void_p),
                                     outV.ctypes.data_as(C.c_void_p)))
            right = outX[:, 0] > p.Lx / 2
            np.multiply(outV, p.np(p.m), out=sV)
            sV[~right] = 0
            LB.check(L.sph_backward(ws.h, tape.h, th.h, C.byref(pc), None,
                                    sV.ctypes.data_as(C.c_void_p), None, 0.2, interval, 64,
                                    C.byref(flags)))
            LB.check(L.sph_workspace_get(ws.h, gX.ctypes.data_as(C.c_void_p),
                                         gV.ctypes.data_as(C.c_void_p),
                                         gth.ctypes.data_as(C.c_void_p)))
            LB.check(L.sph_state_destroy(h))

        solve_host()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            solve_host()
        torch.cuda.synchronize()
        te = (time.perf_counter() - t0) / args.e2e_steps
        h2d = Xh.nbytes + Vh.nbytes + thh.nbytes + Vh.nbytes
        d2h = outX.nbytes + outV.nbytes + gX.nbytes + gV.nbytes + gth.nbytes
        e2e = {"value": N * args.nsteps * world / te, "unit": "particle-steps/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": 1000 * te, "steps": args.e2e_steps,
               "pinned_host_buffers": pinned_ok[0]}

    served = None
    if rank == 0 and world == 1 and args.served and args.workload == "single":
        served = served_sweep(args)

    cpu = None
    if rank == 0 and world == 1 and args.cpu_seconds > 0:
        max_steps = args.nsteps if args.workload == "small" else 64
        cpu = cpu_sample(p_d, X0, V0, theta, args.dtype, budget_s=args.cpu_seconds,
                         max_steps=max_steps, interval=interval)
        cpu.pop("seconds", None)

    if rank == 0:
        line = {"metric": "fwd+adjoint particle-steps/s", "value": value,
                "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
                "data": "synthetic", "config": cfg, "roofline": roof, "cpu_baseline": cpu,
                "e2e": e2e, "gpu_launches": launches, "clocks": clk,
                "solve_roofline": solve_roof, "pass_rooflines": pass_roof,
                "recomputed_forward_steps_per_solve": rec,
                "objective_J": J.value, "kernels_one_solve": kernels,
                "block_sizes": blocks, "fp64_check": fp64, "graph": graph is not None,
                "density_form": args.density_form, "launch_overlap": bool(args.overlap),
                "step_graphs": args.step_graphs, "served": served,
                "graph_kernels_per_solve": graph.nodes if graph is not None else None}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="single",
                    choices=["single", "small", "dense", "batched", "served"])
    ap.add_argument("--served", type=int, default=1,
                    help="single workload: add the served sweep (packed server vs plain) to the "
                         "line")
    ap.add_argument("--requests", type=int, default=100, help="served: requests per rate")
    ap.add_argument("--rates", default="10,100,500", help="served: arrival rates (1/s)")
    ap.add_argument("--served-n", default="2000,200000",
                    help="served: particle-count range of the requests")
    ap.add_argument("--served-steps", default="500,5000",
                    help="served: time-step range of the requests")
    ap.add_argument("--max-inflight", type=int, default=256,
                    help="served: most requests in flight in the packed server")
    ap.add_argument("--hbm-budget-gb", type=float, default=224.0,
                    help="served: admission budget in GiB (of the GPU's 277; the rest holds "
                         "the other workloads' buffers of the same run)")
    ap.add_argument("--instances", type=int, default=64, help="batched: number of instances")
    ap.add_argument("--model", default="reference", choices=sorted(MODELS),
                    help="physics: the reference's (linear EOS, Morris viscosity) or Tait + "
                         "artificial viscosity")
    ap.add_argument("--side", type=int, default=1024, help="lattice side (particles = side^2)")
    ap.add_argument("--nsteps", type=int, default=None,
                    help="time steps per solve (single: 1000; batched: 2000; small and dense "
                         "fix their own)")
    ap.add_argument("--snapshots", type=int, default=None,
                    help="checkpoint slots, 0 = full tape (single: 32; batched: full tape)")
    ap.add_argument("--ntheta", type=int, default=256)
    ap.add_argument("--dtype", default="f32", choices=["f32", "f64"])
    ap.add_argument("--kernel", default="density", choices=sorted(ALGO_WORDS),
                    help="the roofline's kernel (default: the largest share of the solve)")
    ap.add_argument("--kernel-events", type=int, default=0,
                    help="time --kernel with CUDA events inside the timed region (1), or "
                         "(0, default) in a second pass of the same K solves after it: an "
                         "event between two launches breaks their programmatic dependent "
                         "launch and takes whole-solve graphs off, so the headline pass "
                         "carries none")
    ap.add_argument("--traffic-bytes", type=float, default=0.0,
                    help="ncu dram read+write bytes of one launch of --kernel, reported as "
                         "roofline.traffic; 0 = the captured figure at 1,048,576 FP32 "
                         "particles (TRAFFIC_1M_F32), else unknown")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-step-seconds", type=float, default=8.0)
    ap.add_argument("--breakdown", type=int, default=1)
    ap.add_argument("--fp64-check", type=int, default=-1,
                    help="also solve the workload in FP64 on the GPU and report the FP32 "
                         "results' relative difference (the full horizon, and 10 steps of a "
                         "smooth objective); default: on for the single workload")
    ap.add_argument("--density-form", default="pairs", choices=["mask", "tiles", "pairs"],
                    help="FP32 density kernel form: the per-particle mask walk, the cell-tile "
                         "form, or the mask walk with two candidates per iteration (f32x2)")
    ap.add_argument("--overlap", type=int, default=1,
                    help="programmatic dependent launch of the engine's kernels (1) or plain "
                         "stream order (0)")
    ap.add_argument("--step-graphs", type=int, default=32,
                    help="steps that simulate/backward record and replay as one CUDA graph "
                         "(0: launch every kernel on its own)")
    ap.add_argument("--graph", type=int, default=0,
                    help="time replays of the whole solve captured as one CUDA graph")
    ap.add_argument("--autotune", type=int, default=1,
                    help="measure per-kernel block sizes on the workload before timing")
    args = ap.parse_args()
    batched = args.workload == "batched"
    if args.fp64_check < 0:
        args.fp64_check = 1 if args.workload == "single" else 0
    if args.nsteps is None:
        args.nsteps = 2000 if batched else 1000
    if args.snapshots is None:
        args.snapshots = 0 if batched else 32
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "served":
        run_served(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
