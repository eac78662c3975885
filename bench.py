"""Benchmark of the GB300 St-Venant step: FP64 triangle-updates/s on the 1M-triangle case.

Workload: wet/dry flooding over seeded bathymetry, 2 km x 1 km, 1000x500 quads split into
1,000,000 triangles, second-order WAF, per-element lognormal Manning, left-edge inflow
ramping 2 -> 10 m^2/s, fixed 1 m level at the right edge (seeded synthetic inputs stand in
for the reference's real-river meshes, which are not available).

A step is one time step of the whole mesh.  `value` is device-timed throughput with the
state resident in HBM (CUDA events on the solver's stream around K steps replayed from a
CUDA graph); `e2e` times the same metric through the public C ABI with the state copied in
from pinned host memory and read back every step (cf_advance; the three-call sequence
cf_set_state + cf_step + cf_get_state is reported beside it).  The working set (~0.55 GB) is
larger than L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --gpus N > 1 (torchrun) every rank runs its own independent replica ("replicas only":
the plain step on one mesh does not shard across GPUs); value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "FP64 triangle-updates/s @1M tris: plain vs batched; adjoint/forward cost ratio"
UNIT = "tri-updates/s"
# Compulsory HBM bytes per triangle-update of one WAF step: state in and out 48, per-element
# statics 32, neighbour ids 12, per-edge geometry 24 x E/N = 36 (E/N = 1.5), centroids 16.
ALG_BYTES_WAF = 144.0
ALG_BYTES_HLLC = 128.0
# Figures of one ncu capture of this workload's step kernels, keyed by (workload, tuning setting
# (int_compare, int_mul_warps)): DRAM bytes read + written per step (k_edges + k_cells), FP64-pipe
# instructions per edge and per element (DADD + DMUL + DFMA + DSETP + F2F, thread-level, from
# sass__inst_executed_per_opcode), and the FP64-pipe and issue activity ncu reports.  They are
# profile figures, not measured by this run: the bench line carries them under "from_profile" with
# the summary they come from, and only for a (workload, setting) the capture covers.
NCU_PROFILE = {
    ("flooding", (1, 31)): {"traffic": 403.7e6, "fp64_per_edge": 52.9, "fp64_per_element": 16.5,
                            "fp64_pipe": {"k_edges": 0.526, "k_cells": 0.473},
                            "issue": {"k_edges": 0.627, "k_cells": 0.492},
                            "source": "profiles/step_kernels_flooding_1M_WAF.md"},
}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.25)
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.proc is None:
            return
        time.sleep(0.15)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def summary(self):
        if not getattr(self, "rows", None):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def build_case(name: str):
    from cuteflow_gb300 import cases
    if name == "flooding":
        return cases.flooding(1000, 500, seed=2, iflux=3), ALG_BYTES_WAF
    if name == "flooding_muscl":
        return cases.flooding(1000, 500, seed=2, iflux=4), ALG_BYTES_WAF
    if name == "dam_break":
        return cases.circular_dam_break(200, 200, seed=1, iflux=1), ALG_BYTES_HLLC
    raise SystemExit(f"unknown config {name}")


def cpu_baseline(case, budget_s: float = 15.0):
    """Oracle (C++ port of the reference step, OpenMP on all host cores) on a bounded sample:
    the full mesh for as many steps as fit in about budget_s seconds of loop time."""
    from oracle import oracle as O
    O.build()
    threads = O.max_threads()
    probe = O.run(case, 2)
    per_step = max(probe["loop_seconds"] / 2.0, 1e-6)
    k = int(max(2, min(200, budget_s / per_step)))
    r = O.run(case, k)
    rate = case.nelt * k / r["loop_seconds"]
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{k} time steps on the full {case.nelt}-triangle mesh from the initial state "
                      f"({r['loop_seconds']:.2f} s loop time, setup excluded; oracle restating the "
                      f"reference's two-sided per-(element, edge) evaluation)"}


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    case, _ = build_case(args.config)
    from oracle import oracle as O
    O.build()
    threads = O.max_threads()
    probe = O.run(case, 2)
    per_step = max(probe["loop_seconds"] / 2.0, 1e-6)
    budget = 90.0
    k = int(max(1, min(args.steps, budget / per_step)))
    if args.warmup > 0:
        O.run(case, 1)
    r = O.run(case, k)
    rate = case.nelt * k / r["loop_seconds"]
    sample = (f"{k} of the {args.steps} requested time steps on the full {case.nelt}-triangle mesh "
              f"(bounded to ~{budget:.0f} s); oracle = C++ restatement of the reference step "
              f"(two-sided evaluation), OpenMP threads standing in for the reference's MPI ranks")
    line = {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": k,
            "warmup": args.warmup, "ms_per_step": 1e3 * r["loop_seconds"] / k, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": case.name, "triangles": case.nelt, "scheme": {1: "HLLC", 2: "HLLC-Ata", 3: "WAF", 4: "MUSCL-Hancock"}[case.params["iflux"]]},
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def ensemble(nmembers: int, steps: int, warmup: int, seed: int = 3):
    """Batched ensemble vs the same members run one after another through the plain API.

    Members come from the flooding generator (cases.ensemble_member) with seeded sizes (20k-500k
    triangles, skewed to small members) at the benchmark case's 2 m spacing, their own bathymetry,
    lognormal Manning field and inflow peak U(2, 15) m^2/s, WAF.  Both
    forms give bit-identical states, so the comparison is at the same tolerance.  Setup (mesh
    preprocessing, uploads) is excluded from both timings."""
    import torch
    from cuteflow_gb300 import Batch, Solver, cases
    members = [cases.ensemble_member(i, seed=seed) for i in range(nmembers)]
    tri = sum(m.nelt for m in members)
    b = Batch(members)
    for i, m in enumerate(members):
        b.set_state(i, m.U0)
    tune = b.autotune(20)   # the same setting runs in both forms below (results identical in any)
    warm = b.step(warmup, check=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    infos = b.step(steps, check=False)   # a member that stops (the reference's dt-range test) stops alone
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    b.close()
    del b
    t_seq = 0.0
    for m in members:
        s = Solver(m)
        s.set_tuning(tune[0], tune[1])
        s.set_state(m.U0)
        s.step(warmup, check=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.step(steps, check=False)
        torch.cuda.synchronize()
        t_seq += time.perf_counter() - t0
        s.close()
    sizes = sorted(m.nelt for m in members)
    # updates done in the timed steps (a member that stops does fewer)
    tri_steps = sum(m.nelt * (i.steps - w.steps) for m, i, w in zip(members, infos, warm))
    return {"members": nmembers, "steps_each": steps, "triangles_total": tri,
            "triangles_min_median_max": [sizes[0], sizes[len(sizes) // 2], sizes[-1]],
            "batched_value": tri_steps / t_batch, "sequential_value": tri_steps / t_seq,
            "unit": UNIT, "speedup_vs_sequential": t_seq / t_batch,
            "batched_s": t_batch, "sequential_s": t_seq, "stopped_members": sum(1 for i in infos if i.status),
            "stops": [{"member": k, "triangles": members[k].nelt, "status": i.status, "steps": i.steps, "t": i.t,
                       "dt_next": i.dt_next} for k, i in enumerate(infos) if i.status],
            "tuning": {"int_compare": tune[0], "int_mul_warps": tune[1]}}


def ensemble_sizes(steps: int = 200, warmup: int = 10, sizes=(20000, 50000, 100000, 200000, 500000)):
    """Throughput of ensemble-type members by size: one member alone (two members timed, the
    faster kept) against a batch of eight members of that size, both with the tuned setting
    (1, 31).  Members: the flooding generator at the benchmark's 2 m spacing on square domains,
    seeds 500..507.  Shows whether a member run alone is launch- or tail-bound (batching then
    pays) or already fills the GPU."""
    import torch
    from cuteflow_gb300 import Batch, Solver, cases
    rows = []
    for target in sizes:
        ny = int(round(np.sqrt(target / 2.0)))
        nx = int(round(target / 2.0 / ny))
        area = 4.0 * nx * ny
        mem = [cases.flooding(nx, ny, seed=500 + i, lx=2.0 * nx, ly=2.0 * ny, iflux=3,
                              nbumps=max(1, int(round(8.0 * area / 2.0e6))),
                              bump_scale=min(1.0, float(np.sqrt(area / 2.0e6)))) for i in range(8)]
        t_alone = []
        for c in mem[:2]:
            with Solver(c) as s:
                s.set_state(c.U0)
                s.set_tuning(1, 31)
                s.step(warmup)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                s.step(steps)
                torch.cuda.synchronize()
                t_alone.append(time.perf_counter() - t0)
        n = mem[0].nelt
        with Batch(mem) as b:
            for i, c in enumerate(mem):
                b.set_state(i, c.U0)
            b.set_tuning(1, 31)
            b.step(warmup, check=False)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b.step(steps, check=False)
            torch.cuda.synchronize()
            tb = time.perf_counter() - t0
        rows.append({"triangles": n, "wet_fraction": float(np.mean(mem[0].U0[:, 0] > 0)),
                     "alone_ms_per_step": 1e3 * min(t_alone) / steps, "alone_value": n * steps / min(t_alone),
                     "batch8_ms_per_step": 1e3 * tb / steps, "batch8_value": 8 * n * steps / tb,
                     "batched_over_alone": (8 * n * steps / tb) / (n * steps / min(t_alone))})
    return rows


def adjoint_leg(steps: int, warmup: int, obs_every: float = 10.0, budget_gb: float = 64.0):
    """Adjoint Manning calibration: cost of one gradient against one forward.

    Case: 500x200 quads (200,000 triangles) with the circular dam break's flat bed and walls,
    first-order HLLC, true Manning field piecewise constant on 12 seeded Voronoi zones, 40
    seeded gauges observed every 10 s of simulated time.  The gradient is taken at the
    calibration's initial guess n = 0.035 with the objective sum (eta - eta_obs)^2 over the
    observations, with the memory schedule that fits budget_gb of device memory (the recording
    forward keeps the step records of as many of the last steps as fit; the backward replays
    only the others).  Timed with CUDA events on the solver's stream:
      forward   : N plain steps (cf_step),
      record    : the recording forward (cf_adjoint_forward: steps + gauges + records/checkpoints),
      backward  : cf_adjoint_backward (replays of the checkpointed steps + reverse steps).
    ratio = (record + backward) / forward, the cost of a gradient in forward runs.  The same
    gradient with the sqrt(N) checkpoint schedule (no budget) is timed beside it."""
    import torch
    from cuteflow_gb300 import Solver, cases
    from cuteflow_gb300.adjoint import Adjoint, zone_gradient
    c, zones, nz_true, gauges = cases.calibration()
    n0 = np.full(c.nelt, 0.035)
    s = Solver(c)
    s.set_state(c.U0)
    tune = s.autotune(20)   # the forward, the recording forward and the replays all run this setting
    stream = torch.cuda.ExternalStream(s.stream())
    adj = Adjoint(s, steps, gauges, 0, budget_bytes=int(budget_gb * (1 << 30)))

    def timed(fn):
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = fn()
        b.record(stream)
        torch.cuda.synchronize()
        return out, a.elapsed_time(b)

    # observations from the true field
    s.set_manning(c.manning)
    s.set_state(c.U0)
    eta_obs, _ = adj.forward()
    dt, t = adj.dt_history()
    obs = cases.observation_steps(t, dt, obs_every)
    # calibration guess: warm-up, then the timed legs
    s.set_manning(n0)
    s.set_state(c.U0)
    s.step(warmup)
    s.set_state(c.U0)
    _, fwd_ms = timed(lambda: s.step(steps))
    s.set_state(c.U0)
    adj.forward()
    s.set_state(c.U0)
    (eta, _), rec_ms = timed(lambda: adj.forward())
    w = np.zeros_like(eta)
    w[obs] = 2.0 * (eta[obs] - eta_obs[obs])
    misfit = float(np.sum((eta[obs] - eta_obs[obs]) ** 2))
    adj.backward(w)
    (gU, gn), bwd_ms = timed(lambda: adj.backward(w))
    gz = zone_gradient(gn, zones, nz_true.size)
    ok = bool(np.isfinite(gn).all() and np.isfinite(gU).all())
    sched = dict(adj.schedule)
    adj.close()
    # the sqrt(N) checkpoint schedule: same gradient, one replay of every step in the backward
    with Adjoint(s, steps, gauges, 0) as a2:
        s.set_state(c.U0)
        (_, _), rec2_ms = timed(lambda: a2.forward())
        (gU2, gn2), bwd2_ms = timed(lambda: a2.backward(w))
        same = bool(np.array_equal(gn2, gn) and np.array_equal(gU2, gU))
        sched2 = dict(a2.schedule)
    out = {"workload": c.name, "triangles": c.nelt, "scheme": "HLLC", "steps": steps,
           "schedule": sched, "budget_gb": budget_gb, "gauges": int(gauges.size),
           "observations": int(obs.size), "device_bytes": sched["device_bytes"],
           "forward_ms": fwd_ms, "record_ms": rec_ms, "backward_ms": bwd_ms,
           "ratio": (rec_ms + bwd_ms) / fwd_ms, "ratio_target": 5.0,
           "forward_value": c.nelt * steps / (fwd_ms * 1e-3),
           "gradient_value": c.nelt * steps / ((rec_ms + bwd_ms) * 1e-3), "unit": UNIT,
           "misfit": misfit, "zone_gradient": [float(x) for x in gz],
           "zones_with_zero_gradient": int(np.sum(gz == 0.0)), "finite": ok,
           "sqrt_schedule": {"schedule": sched2, "record_ms": rec2_ms, "backward_ms": bwd2_ms,
                             "ratio": (rec2_ms + bwd2_ms) / fwd_ms, "gradient_bit_identical": same},
           "tuning": {"int_compare": tune[0], "int_mul_warps": tune[1]}}
    s.close()
    return out


def budget_groups(nelts, steps: int, budget: int):
    """Consecutive instances packed into groups whose adjoint fits budget bytes with every step
    record stored: 80 bytes per element and step (state and flux sums) plus ~400 bytes per element
    of step buffers, slots, edge tables and checkpoints, with 2 % of slack.  An instance that does
    not fit alone forms its own group (its adjoint then replays part of its steps)."""
    per = lambda n: int(1.02 * n * (80 * steps + 400)) + (64 << 20)
    groups, cur, used = [], [], 0
    for i, n in enumerate(nelts):
        if cur and used + per(n) > budget:
            groups.append(cur)
            cur, used = [], 0
        cur.append(i)
        used += per(n)
    if cur:
        groups.append(cur)
    return groups


def calibration_batch_leg(ninst: int, steps: int, iters: int, obs_every: float = 10.0, full: bool = False,
                          budget_gb: float = 120.0, seq_iters: int = 1, fd_zones: int = 0):
    """Batched adjoint calibration: ninst instances of the calibration case with seeded sizes, zone
    fields and gauges.  Instances are packed, in order, into groups whose adjoint step records fit
    budget_gb of device memory together (budget_groups), so that no group replays a step; each
    group is one batch context, and every gradient-descent iteration runs one recording forward
    and one backward for the group's instances in the same launches, sums dJ/dn per zone and
    steps the zone values on the device (the instances are independent calibrations, so the
    groups run one after another, each for all iterations, with the learning rate of its first
    gradient).  Timed against the same instances' one-member adjoints run one after another
    (forward, backward, zone gradient and step each, with the same cap).  Misfit: sum of squared
    gauge misfits every obs_every s, summed over the instances.  Instance meshes: 8k-39k triangles
    for the sample, 50k-273k with full (the workload's sizes); observations every 10 s with full,
    every 1 s for the sample (its 400 steps cover a few seconds).  The one-after-another form runs
    seq_iters iterations per instance (its time per iteration does not depend on the
    iteration)."""
    import torch
    from cuteflow_gb300 import Batch, Solver, cases
    from cuteflow_gb300.adjoint import Adjoint, Zones
    if not full:
        obs_every = min(obs_every, 1.0)
    inst = []
    for i in range(ninst):
        if full:
            nx, ny = int(250 + (i * 37) % 300), int(100 + (i * 23) % 180)
        else:
            nx, ny = int(100 + (i * 37) % 120), int(40 + (i * 23) % 50)
        c, zones, nz, gauges = cases.calibration(nx, ny, seed=10 + i, nzones=8 + i % 9, ngauges=20 + (i * 7) % 41)
        inst.append((c, zones, nz, gauges))
    tri = sum(c.nelt for c, *_ in inst)
    zoff = np.cumsum([0] + [len(nz) for _, _, nz, _ in inst])
    true_vals = np.concatenate([nz for _, _, nz, _ in inst])
    gg = np.concatenate([g for *_, g in inst]).astype(np.int32)
    budget = int(budget_gb * (1 << 30))
    groups = budget_groups([c.nelt for c, *_ in inst], steps, budget)
    vals0 = np.full(int(zoff[-1]), 0.035)
    vals = vals0.copy()
    eta_obs_i, mask_i, lr_i = [None] * ninst, [None] * ninst, [None] * ninst
    misfits = np.zeros(iters + 1)
    t_batch, scheds, fd = 0.0, [], []
    for gi, grp in enumerate(groups):
        # one batch context per group: its adjoint's step records fit the budget (nothing replayed)
        zl = np.concatenate([inst[i][1] + (zoff[i] - zoff[grp[0]]) for i in grp])
        gmg = np.concatenate([np.full(len(inst[i][3]), k, np.int32) for k, i in enumerate(grp)])
        ggg = np.concatenate([inst[i][3] for i in grp]).astype(np.int32)
        z_lo, z_hi = int(zoff[grp[0]]), int(zoff[grp[-1] + 1])
        b = Batch([inst[i][0] for i in grp])
        adj = Adjoint(b, steps, ggg, 0, gauge_member=gmg, budget_bytes=budget)
        scheds.append({"instances": len(grp), "triangles": int(sum(inst[i][0].nelt for i in grp)), **adj.schedule})
        zs = Zones(b, zl.astype(np.int32), z_hi - z_lo)

        def start():
            for k, i in enumerate(grp):
                b.set_state(k, inst[i][0].U0)

        zs.set(true_vals[z_lo:z_hi])
        start()
        eta_obs, _ = adj.forward()
        dt, t = adj.dt_history()
        dt, t = dt.reshape(steps, -1), t.reshape(steps, -1)
        gcol = np.cumsum([0] + [len(inst[i][3]) for i in grp])
        mask = np.zeros_like(eta_obs)
        for k, i in enumerate(grp):
            mask[cases.observation_steps(t[:, k], dt[:, k], obs_every), gcol[k]:gcol[k + 1]] = 1.0
            eta_obs_i[i], mask_i[i] = eta_obs[:, gcol[k]:gcol[k + 1]], mask[:, gcol[k]:gcol[k + 1]]
        zs.set(vals0[z_lo:z_hi])
        lr = None
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for it in range(iters):
            start()
            eta, _ = adj.forward()
            r = (eta - eta_obs) * mask
            misfits[it] += float(np.sum(r * r))
            adj.backward(2.0 * r)
            g = zs.gradient(adj)
            if lr is None:
                lr = 0.004 / max(np.abs(g).max(), 1e-300)
            zs.descend(lr, 0.01, 0.1)
        torch.cuda.synchronize()
        t_batch += (time.perf_counter() - t0) / iters
        for i in grp:
            lr_i[i] = lr
        start()
        eta, _ = adj.forward()
        r = (eta - eta_obs) * mask
        misfits[iters] += float(np.sum(r * r))
        vals[z_lo:z_hi] = zs.get()[0]
        # central differences (step 1e-6 relative, the recorded dt sequence replayed) of the first
        # group's zones with the largest gradients at the final values, against its zone gradient
        if gi == 0 and fd_zones > 0:
            adj.backward(2.0 * r)
            g = zs.gradient(adj)
            vg = vals[z_lo:z_hi]
            for z in np.argsort(-np.abs(g))[:fd_zones]:
                d = 1e-6 * vg[z]
                Jz = []
                for sign in (1.0, -1.0):
                    v = vg.copy()
                    v[z] += sign * d
                    zs.set(v)
                    start()
                    e_, _ = adj.forward(replay=True)
                    Jz.append(((e_ - eta_obs) * mask))
                zs.set(vg)
                dJ = float(np.sum((Jz[0] - Jz[1]) * (Jz[0] + Jz[1])))
                fdz = dJ / (2.0 * d)
                fd.append({"zone": int(z_lo + z), "adjoint": float(g[z]), "central_difference": fdz,
                           "relative_difference": abs(fdz - g[z]) / abs(g[z])})
        zs.close(); adj.close(); b.close()
    # the same iteration, instance by instance
    t_seq = 0.0
    for i, (c, zones, nz, gauges) in enumerate(inst):
        s = Solver(c)
        a1 = Adjoint(s, steps, gauges, 0, budget_bytes=budget)
        z1 = Zones(s, zones, len(nz))
        z1.set(vals0[zoff[i]:zoff[i + 1]])
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for it in range(seq_iters):
            s.set_state(c.U0)
            eta_i, _ = a1.forward()
            a1.backward(2.0 * (eta_i - eta_obs_i[i]) * mask_i[i])
            z1.gradient(a1)
            z1.descend(lr_i[i], 0.01, 0.1)
        torch.cuda.synchronize()
        t_seq += (time.perf_counter() - t1) / seq_iters
        z1.close(); a1.close(); s.close()
    return {"instances": ninst, "triangles_total": tri, "steps": steps, "iterations": iters,
            "budget_gb": budget_gb, "groups": scheds, "observation_every_s": obs_every,
            "zones_total": int(zoff[-1]), "gauges_total": int(gg.size),
            "batched_s_per_iteration": t_batch, "sequential_s_per_iteration": t_seq,
            "sequential_iterations_timed": seq_iters,
            "speedup_vs_sequential": t_seq / t_batch, "misfit_per_iteration": [float(m) for m in misfits],
            "zone_error_start": float(np.abs(vals0 - true_vals).mean()),
            "zone_error_end": float(np.abs(vals - true_vals).mean()), "fd_check": fd}


def run_ours(args):
    import torch
    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        pg = dist
    from cuteflow_gb300 import Solver, build
    build.build()
    case, alg_bytes = build_case(args.config)
    n = case.nelt
    s = Solver(case)
    stream = torch.cuda.ExternalStream(s.stream())

    def barrier():
        torch.cuda.synchronize()
        if pg is not None:
            pg.barrier()

    # ---- autotuner: how the edge kernel shares FP64 work with the integer pipes (identical
    # results in every setting); the trials run on the initial state, which is restored ----
    s.set_state(case.U0)
    if args.tuning:
        cmp_, mask = (int(v) for v in args.tuning.split(","))
        s.set_tuning(cmp_, mask)
        tune = (cmp_, mask, None)
    else:
        tune = s.autotune(30) if not args.no_tune else (0, 0, None)

    # the launch shapes the autotuner chose among, each timed on the same state (20 steps), then the
    # chosen one restored
    shape = s.launch_shape()
    shape_ms = {}
    for eb in ((64, 128, 256) if not args.no_shape_sweep else ()):
        for ept in (1, 2):
            for cb in (256, 128):
                s.set_launch_shape(eb, ept, cb)
                s.set_state(case.U0)
                s.step(3)
                torch.cuda.synchronize()
                a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a0.record(stream)
                s.step(20)
                a1.record(stream)
                torch.cuda.synchronize()
                shape_ms[f"{eb}x{ept}/{cb}"] = a0.elapsed_time(a1) / 20
    s.set_launch_shape(*shape)

    # ---- device-resident throughput (value) ----
    s.set_state(case.U0)
    s.step(args.warmup)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        e0.record(stream)
        info = s.step(args.steps)
        e1.record(stream)
        barrier()
    ms = e0.elapsed_time(e1)
    # the dry parts of the mesh take the kernels' dry-region shortcuts, so the step's cost depends on
    # how much of the mesh is wet: reported at the start and at the end of the timed steps
    wet_end = float(np.mean(s.get_state()[:, 0] > 0.0))
    wet_start = float(np.mean(case.U0[:, 0] > 0.0))
    if pg is not None:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
    value = world * n * args.steps / (ms * 1e-3)

    # ---- per-kernel durations of the same workload (events around each kernel) ----
    ksteps = min(args.steps, 200)
    s.set_timing(True)
    s.step(ksteps)
    s.set_timing(False)
    flux_ms, upd_ms, launches = s.timing()
    k_edges_ms = flux_ms / ksteps
    k_cells_ms = upd_ms / ksteps
    step_kernel_ms = k_edges_ms + k_cells_ms

    # ---- end to end through the C ABI with host buffers ----
    e2e_steps = min(args.steps, 50)
    hin = torch.from_numpy(np.ascontiguousarray(case.U0)).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    import ctypes
    from cuteflow_gb300 import _abi
    lib = s._L
    dp = ctypes.POINTER(ctypes.c_double)
    pin_in = ctypes.cast(hin.data_ptr(), dp)
    pin_out = ctypes.cast(hout.data_ptr(), dp)
    stepinfo = _abi.CfStepInfo()
    lib.cf_set_state(s._ctx, pin_in, 0.0)
    lib.cf_step(s._ctx, 1, ctypes.byref(stepinfo))
    barrier()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for _ in range(e2e_steps):
        rc = lib.cf_set_state(s._ctx, pin_in, 0.0)
        rc |= lib.cf_step(s._ctx, 1, ctypes.byref(stepinfo))
        rc |= lib.cf_get_state(s._ctx, pin_out)
        if rc:
            raise SystemExit("C ABI call failed during the e2e loop")
    f1.record(stream)
    barrier()
    three_ms = f0.elapsed_time(f1)
    # the same per step through cf_advance: state in, one step, state out, one wait
    def advance_ms():
        lib.cf_advance(s._ctx, pin_in, 0.0, 1, pin_out, ctypes.byref(stepinfo))
        barrier()
        f0.record(stream)
        for _ in range(e2e_steps):
            if lib.cf_advance(s._ctx, pin_in, 0.0, 1, pin_out, ctypes.byref(stepinfo)):
                raise SystemExit("C ABI call failed during the e2e loop")
        f1.record(stream)
        barrier()
        return f0.elapsed_time(f1)

    # the same calls with every state buffer staged through the device copy (cf_set_direct_io 0),
    # then the default: the state kernels read and write the pinned buffers over the CPU link
    s.set_direct_io(False)
    staged_ms = advance_ms()
    s.set_direct_io(True)
    e2e_ms = advance_ms()
    if pg is not None:
        t = torch.tensor([e2e_ms, three_ms, staged_ms], device="cuda", dtype=torch.float64)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        e2e_ms, three_ms, staged_ms = float(t[0].item()), float(t[1].item()), float(t[2].item())
    e2e_value = world * n * e2e_steps / (e2e_ms * 1e-3)
    three_value = world * n * e2e_steps / (three_ms * 1e-3)
    staged_value = world * n * e2e_steps / (staged_ms * 1e-3)
    # the host link's own rate for the same bytes (plain pinned copies, no kernels): the floor of
    # the end-to-end step's copy time
    dbuf = torch.empty(hin.numel(), dtype=torch.float64, device="cuda")
    hv, ho = hin.view(-1), hout.view(-1)

    def link_ms(fn, k=10):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(k):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / k

    h2d_ms = link_ms(lambda: dbuf.copy_(hv, non_blocking=True))
    d2h_ms = link_ms(lambda: ho.copy_(dbuf, non_blocking=True))
    del dbuf

    hbm, hbm_src = peaks()
    achieved = alg_bytes * n / (step_kernel_ms * 1e-3) / 1e9
    fp64_rate = s.probe_fp64()
    prof = NCU_PROFILE.get((args.config, (tune[0], tune[1])))
    fp64_instr = None
    if prof:
        fp64_instr = prof["fp64_per_edge"] * s.nedge + prof["fp64_per_element"] * n
    fp64_achieved = fp64_instr / (step_kernel_ms * 1e-3) if fp64_instr else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generator with the benchmark case's shapes and distributions)",
        "config": {"workload": case.name, "triangles": n, "edges": s.nedge,
                   "scheme": {1: "HLLC", 2: "HLLC-Ata", 3: "WAF", 4: "MUSCL-Hancock"}[case.params["iflux"]],
                   "l2": "working set > L2 (no flush needed)", "parallelism": f"replicas x{world}",
                   "time_steps_ran": info.steps,
                   "wet_fraction": {"start": wet_start, "end_of_timed_steps": wet_end},
                   "tuning": {"int_compare": tune[0], "int_mul_warps": tune[1], "trial_ms_per_step": tune[2],
                              "launch_shape": {"edge_block": shape[0], "edges_per_thread": shape[1],
                                               "cell_block": shape[2]},
                              "ms_per_step_by_shape": shape_ms}},
        "roofline": {"bound": "hbm", "kernel": "one time step (k_edges + k_cells)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({hbm_src})",
                     "alg_bytes_per_tri": alg_bytes,
                     "traffic": prof["traffic"] if prof else None,
                     "traffic_note": ("from_profile: ncu dram__bytes_read.sum + dram__bytes_write.sum per step "
                                      "(k_edges + k_cells) of this workload and setting, " + prof["source"])
                                     if prof else "no ncu capture of this workload and setting",
                     "k_edges_ms": k_edges_ms, "k_cells_ms": k_cells_ms},
        "fp64": {"peak_instr_per_s": fp64_rate,
                 "peak_source": "cf_probe_fp64, measured live: independent FMA chains on every SM",
                 "instr_per_step": fp64_instr,
                 "achieved_instr_per_s": fp64_achieved,
                 "frac": fp64_achieved / fp64_rate if fp64_achieved else None,
                 "from_profile": ({"source": prof["source"], "fp64_per_edge": prof["fp64_per_edge"],
                                   "fp64_per_element": prof["fp64_per_element"],
                                   "fp64_pipe_active": prof["fp64_pipe"], "issue_active": prof["issue"]}
                                  if prof else None),
                 "note": "instr_per_step is the profile's FP64-pipe instruction count of this workload and "
                         "setting; achieved divides it by the live kernel time"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 24 * n,
                "steps": e2e_steps, "ms_per_step": e2e_ms / e2e_steps,
                "link_h2d_gbs": 24 * n / (h2d_ms * 1e-3) / 1e9, "link_d2h_gbs": 24 * n / (d2h_ms * 1e-3) / 1e9,
                "three_calls_value": three_value, "three_calls_ms_per_step": three_ms / e2e_steps,
                "staged_value": staged_value, "staged_ms_per_step": staged_ms / e2e_steps,
                "note": "per step: cf_advance (the state from pinned host memory, one step, the state back "
                        "into pinned host memory, one wait), the state kernels reading and writing the pinned "
                        "buffers over the CPU link; staged: the same with cudaMemcpyAsync copies through a "
                        "device staging buffer (cf_set_direct_io 0); three_calls: cf_set_state + cf_step + "
                        "cf_get_state; link_*: plain pinned copies of the same bytes"},
        "gpu_launches": 2 * args.steps + 1,
        "clocks": clk.summary(),
    }
    if rank == 0 and args.batched_members > 0:
        line["batched"] = ensemble(args.batched_members, args.batched_steps, 3)
        line["batched"]["note"] = ("sample of the 256-member, 2000-step ensemble workload; run "
                                   "`bench.py --config ensemble` for the full size")
    if rank == 0 and args.adjoint_steps > 0:
        line["adjoint"] = adjoint_leg(args.adjoint_steps, 10, budget_gb=args.adjoint_budget_gb)
    if rank == 0 and args.calib_instances > 0:
        line["batched_adjoint"] = calibration_batch_leg(args.calib_instances, args.calib_steps, args.calib_iters,
                                                        full=args.calib_full, budget_gb=args.calib_budget_gb,
                                                        seq_iters=args.calib_seq_iters, fd_zones=args.calib_fd_zones)
        line["batched_adjoint"]["note"] = (
            "the 64-instance calibration workload's instance sizes (50k-273k triangles)" if args.calib_full else
            "sample of the 64-instance calibration workload (50k-300k triangles, 3000 steps, 10 iterations); "
            "`--calib-instances 64 --calib-steps 3000 --calib-full` runs its sizes")
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(case)
    s.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="flooding", choices=["flooding", "flooding_muscl", "dam_break", "ensemble", "ensemble_sizes"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-tune", action="store_true", help="skip the autotuner (every operation on the FP64 pipe)")
    ap.add_argument("--no-shape-sweep", action="store_true",
                    help="do not time every launch shape beside the chosen one (the profiling commands use it)")
    ap.add_argument("--tuning", default=None, metavar="CMP,MASK",
                    help="fix the edge kernel's integer-pipe setting instead of autotuning (e.g. 1,15)")
    ap.add_argument("--batched-members", type=int, default=32, help="ensemble sample beside the plain line (0: skip)")
    ap.add_argument("--batched-steps", type=int, default=200)
    ap.add_argument("--calib-instances", type=int, default=8, help="batched calibration leg (0: skip)")
    ap.add_argument("--calib-steps", type=int, default=400)
    ap.add_argument("--calib-iters", type=int, default=3)
    ap.add_argument("--calib-full", action="store_true", help="calibration instances at the workload's sizes")
    ap.add_argument("--calib-budget-gb", type=float, default=120.0, help="device memory cap of the batch's adjoint")
    ap.add_argument("--calib-fd-zones", type=int, default=2,
                    help="central-difference check of the batch's zone gradient on this many zones")
    ap.add_argument("--calib-seq-iters", type=int, default=1,
                    help="iterations of the one-after-another comparison per instance")
    ap.add_argument("--adjoint-budget-gb", type=float, default=64.0, help="device memory cap of the adjoint leg")
    ap.add_argument("--adjoint-steps", type=int, default=3000,
                    help="adjoint calibration leg beside the plain line (0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.config == "ensemble_sizes":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        from cuteflow_gb300 import build
        build.build()
        rows = ensemble_sizes()
        print(json.dumps({"metric": "ensemble member throughput by size: " + METRIC, "unit": UNIT, "n_gpus": 1,
                          "dtype": "f64", "data": "synthetic", "rows": rows}), flush=True)
        return
    if args.config == "ensemble":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        from cuteflow_gb300 import build
        build.build()
        r = ensemble(args.batched_members if args.batched_members > 32 else 256, args.steps, args.warmup)
        print(json.dumps({"metric": "batched ensemble: " + METRIC, "value": r["batched_value"], "unit": UNIT,
                          "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                          "dtype": "f64", "data": "synthetic", "config": {"workload": "ensemble_256_waf"},
                          "batched": r}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
