#!/usr/bin/env python
"""Benchmark of the coupled free-surface LB / DEM impact step on GB300.

One "step" is one goCycle of the reference (DEM step, coupling step, LB
step, free-surface step) on the configured workload. ``value`` is the
coupled MLUPS (active-node updates per second over the whole cycle) with the
run resident in HBM; ``e2e`` is the same metric through the C ABI from host
inputs (case upload, per-step impactor read-back). ``roofline`` covers the
dominant kernel (the fused collide+stream lattice kernel), timed live with
CUDA events on the stream it runs on. ``cpu_baseline`` times the CPU
restatement of the reference algorithm on a bounded sample of the same
workload.

usage: python bench.py [--gpus N] [--steps K] [--warmup W]
                       [--impl ours|reference] [--precision mixed|fp64]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

# Many runs share the GPU through their own streams; the CUDA driver maps streams
# onto this many hardware work queues (default 8), so more than 8 runs would
# wait on one another's queues. Must be set before the CUDA context exists.
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "lbm-dem_gb300"))
sys.path.insert(0, os.path.join(REPO, "tests"))

CACHE = os.path.join(REPO, "bench_cache")
WORKLOADS = {
    "c2": "256x320x256 lattice (y vertical) filled to y=240, 25000 bidisperse spheres "
          "(r 3.0/4.2) randomly inserted and compressed into a bed of volume fraction 0.50 "
          "(164 high), impactor r=20 density 5 vy=-0.02, tau=0.6",
    "c1": "64x80x64 lattice filled to y=60, 400 bidisperse spheres (r 3.0/4.2, seeded RSA), "
          "impactor r=8 density 5 vy=-0.01, tau=0.8",
    "c2s": "160x200x160 lattice filled to y=150, 6100 bidisperse spheres (r 3.0/4.2) in a "
           "compressed bed of volume fraction 0.50, impactor r=14 density 5 vy=-0.02, tau=0.6 "
           "(profiling size of c2)",
    "c5": "512x384x512 lattice filled to y=300, 200000 bidisperse spheres (r 3.0/4.2) "
          "randomly inserted and compressed into a bed of volume fraction 0.55 (296 high), "
          "impactor r=32 density 8 vy=-0.03, tau=0.6",
}
# Algorithmic bytes per active-node update of the lattice kernel: 19
# populations read + 19 written, 8 B (plain FP64) or 4 B (FP32 storage).
BYTES_PER_NODE = {"fp64": 304, "mixed": 152}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def case_path(workload: str) -> str:
    import casegen
    d = os.path.join(CACHE, workload)
    cfg = os.path.join(d, "parameters.cfg")
    if not os.path.exists(cfg):
        log(f"generating workload {workload} ...")
        casegen.named_case(workload).write(d)
    return cfg


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            j = json.load(fh)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(CACHE, f"clocks_{os.getpid()}.csv")

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.proc.terminate()
        self.proc.wait()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.remove(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v: float) -> float:
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allsum(world, v: float) -> float:
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], device="cuda", dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def upload_bytes(cfg) -> int:
    """Bytes lbdem_create copies from the host: the particle and impactor
    tables and the small run records (the lattice itself is initialised on the
    device from the configuration)."""
    c = cfg.cfg
    P, O = c.n_particles, c.n_objects
    return int(P * 8 * (3 + 1 + 1 + 1 + 3) + max(O, 1) * 44 * 8 + 6 * 48 + 6 * 4 + 6 * 4 + 8
               + 32 * 4)


def bench_config(args, cfg, world) -> dict:
    """The ``config`` of both arms' lines, from the case itself (identical for
    the GPU arm and the reference arm)."""
    c = cfg.cfg
    L = float(c.unitLength)
    lattice = [int(math.floor(v / L + 0.5)) for v in (c.lbSizeX, c.lbSizeY, c.lbSizeZ)]
    nodes = lattice[0] * lattice[1] * lattice[2]
    gb = nodes * 19 * 4 / 1e9  # one FP32 population lattice
    l2 = (f"one population lattice is {gb:.2f} GB, larger than the 129 MB L2: no flush"
          if gb > 0.129 else
          f"one population lattice is {gb * 1e3:.0f} MB, within the 129 MB L2: "
          f"kernel times are L2-assisted")
    return {"workload": args.workload, "description": WORKLOADS[args.workload],
            "lattice": lattice, "particles": int(c.n_particles),
            "parallelism": f"replicas{world}", "l2": l2}


PORT_KIND = ("port: the oracle, a dense-array restatement of the reference's step "
             "(bit-exact against the compiled reference); faster than the reference's own "
             "node-list code, so the ratio against it understates the speed-up over the "
             "reference itself")


def cpu_baseline(cfg, workload, steps, warm=1, budget_s=75.0, single_s=30.0) -> dict:
    """The oracle (CPU restatement of the reference algorithm, OpenMP on its
    per-node loops) on a bounded sample of the workload: up to ``steps``
    coupled steps on all host threads within ``budget_s``, then a one-thread
    figure on up to ``single_s`` of further steps."""
    import oracle_ffi
    oracle_ffi.build_oracle()
    cores = oracle_ffi.max_threads()
    orc = oracle_ffi.Oracle(cfg)
    orc.cycle(warm)

    def timed(limit_steps, limit_s):
        done, upd, t0 = 0, 0, time.perf_counter()
        while done < limit_steps and (done == 0 or time.perf_counter() - t0 < limit_s):
            orc.cycle(1)
            upd += orc.counters()[3]
            done += 1
        return done, upd, time.perf_counter() - t0

    done, upd, dt = timed(steps, budget_s)
    oracle_ffi.set_threads(1)
    d1, u1, t1 = timed(steps, single_s)
    oracle_ffi.set_threads(cores)
    orc.close()
    return {"value": round(upd / dt / 1e6, 4), "unit": "MLUPS", "cores": cores,
            "kind": "port",
            "sample": f"{done} coupled steps of workload {workload} (of {steps} asked, "
                      f"{budget_s:.0f} s budget) after {warm} warm-up step(s), {cores} threads; "
                      + PORT_KIND,
            "single_thread": {"value": round(u1 / t1 / 1e6, 4), "unit": "MLUPS",
                              "steps": d1, "cores": 1}}


def run_reference(args, world, rank):
    """Reference arm: the CPU restatement of the reference's algorithm (the
    oracle; the reference itself cannot be built on the GPU host), timed on
    the host's cores. Reads the case with the pure-Python reader, so nothing
    but the oracle's library is loaded."""
    if rank != 0:
        return
    import caseio
    cfg = caseio.CaseConfig(case_path(args.workload))
    cb = cpu_baseline(cfg, args.workload, steps=args.steps, warm=min(args.warmup, 1),
                      budget_s=150.0)
    line = {"impl": "reference", "metric": "coupled MLUPS", "value": cb["value"],
            "unit": "MLUPS", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": bench_config(args, cfg, world),
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": "MLUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def kernel_roofline(prof, precision: str) -> dict:
    """The lattice kernel's own figure from its CUDA-event time per launch."""
    peak, peak_kind = peaks()
    bpn = BYTES_PER_NODE[precision]
    achieved = bpn * prof.active_node_updates / (prof.lb_kernel_ms * 1e-3) / 1e9 \
        if prof.lb_kernel_ms > 0 else 0.0
    return {"achieved": round(achieved, 1), "peak": peak, "peak_kind": peak_kind,
            "frac": round(achieved / peak, 4), "bytes_per_active_node": bpn,
            "kernel_ms_per_launch": round(prof.lb_kernel_ms / max(prof.lb_kernel_launches, 1), 4)}


def timed_cycles(solver, n: int, torch, stream) -> tuple[float, object]:
    """n goCycles between CUDA events on the run's stream; (ms, counters)."""
    solver.sync()
    solver.profile_read(reset=True)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    solver.cycle(n)
    ev1.record(stream)
    torch.cuda.synchronize()
    solver.sync()
    return ev0.elapsed_time(ev1), solver.profile_read(reset=True)


def late_window(args, cfg, local, torch) -> dict:
    """The mixed form after the impact: a fresh run advanced to cycle
    ``--late-start``, then ``--late-steps`` cycles timed (neighbour-list
    rebuilds nearly every step, impactor coupled to the suspension)."""
    import lbdem
    sv = lbdem.Solver(cfg, precision=lbdem.MIXED, device=local)
    st = torch.cuda.Stream(device=local)
    sv.set_stream(st.cuda_stream)
    sv.cycle(args.late_start)
    r0 = sv.get_info().neighbour_rebuilds
    ms, p = timed_cycles(sv, args.late_steps, torch, st)
    r1 = sv.get_info().neighbour_rebuilds
    sv.profile_enable(True)
    sv.cycle(args.late_steps)
    sv.sync()
    prof = sv.profile_read(reset=True)
    sv.close()
    return {"cycles": [args.late_start + 1, args.late_start + args.late_steps],
            "value": round(p.active_node_updates / (ms * 1e-3) / 1e6, 2), "unit": "MLUPS",
            "ms_per_step": round(ms / args.late_steps, 4),
            "neighbour_rebuilds": int(r1 - r0),
            "lattice_kernel": kernel_roofline(prof, "mixed")}


def fp64_form(args, cfg, local, torch) -> dict:
    """The plain FP64 form (the parity form) on the same workload."""
    import lbdem
    sv = lbdem.Solver(cfg, precision=lbdem.PLAIN_FP64, device=local)
    st = torch.cuda.Stream(device=local)
    sv.set_stream(st.cuda_stream)
    sv.cycle(max(args.warmup, 3))
    ms, p = timed_cycles(sv, args.fp64_steps, torch, st)
    sv.profile_enable(True)
    sv.cycle(min(args.fp64_steps, 10))
    sv.sync()
    prof = sv.profile_read(reset=True)
    sv.close()
    k = kernel_roofline(prof, "fp64")
    k["bound"] = ("FP64 pipe: about 600 FP64 operations per node with the reference's "
                  "divides; the HBM fraction above is not its limit")
    return {"steps": args.fp64_steps, "value": round(p.active_node_updates / (ms * 1e-3) / 1e6, 2),
            "unit": "MLUPS", "ms_per_step": round(ms / args.fp64_steps, 4),
            "lattice_kernel": k}


def run_ours(args, world, rank, local):
    import torch
    import lbdem
    torch.cuda.set_device(local)
    prec = lbdem.MIXED if args.precision == "mixed" else lbdem.PLAIN_FP64
    cfg = lbdem.LoadedConfig(case_path(args.workload))
    K, W = args.steps, args.warmup

    # ---- device-resident timed region ----
    solver = lbdem.Solver(cfg, precision=prec, device=local)
    stream = torch.cuda.Stream(device=local)
    solver.set_stream(stream.cuda_stream)
    solver.cycle(W)
    solver.sync()
    solver.profile_read(reset=True)
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    ev0.record(stream)
    solver.cycle(K)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    solver.sync()
    ms = ev0.elapsed_time(ev1)
    timed = solver.profile_read(reset=True)
    ms_max = allmax(world, ms)
    upd_all = allsum(world, float(timed.active_node_updates))
    value = upd_all / (ms_max * 1e-3) / 1e6
    # the lattice kernel's own time (roofline): CUDA events around each of its
    # launches, in K further cycles (the events keep the cycles from being
    # replayed as CUDA graphs, so they are not the timed region above)
    solver.profile_enable(True)
    solver.cycle(K)
    solver.sync()
    prof = solver.profile_read(reset=True)
    solver.profile_enable(False)
    solver.close()

    # ---- end to end through the C ABI: case upload, K cycles, per-step read-back ----
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s2 = lbdem.Solver(cfg, precision=prec, device=local)
    s2.profile_read(reset=True)
    for _ in range(K):
        s2.cycle(1)
        s2.objects()  # impactor state back to the host every step
    p2 = s2.profile_read(reset=True)
    t_e2e = time.perf_counter() - t0
    n_obj = int(s2.get_info().n_objects)
    s2.close()
    e2e_val = allsum(world, float(p2.active_node_updates)) / allmax(world, t_e2e) / 1e6

    kr = kernel_roofline(prof, args.precision)
    traffic = None
    tr = os.path.join(REPO, "profiles", f"traffic_{args.precision}.json")
    if os.path.exists(tr):
        with open(tr) as fh:
            t = json.load(fh)
        if prof.lb_kernel_launches:
            # bytes per active node from the ncu capture, scaled to this launch
            traffic = t["dram_bytes_per_active_node"] * prof.active_node_updates / \
                prof.lb_kernel_launches
    if rank != 0:
        return
    up = upload_bytes(cfg)
    extra = world == 1
    line = {
        "metric": "coupled MLUPS", "value": round(value, 2), "unit": "MLUPS",
        "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": round(ms_max / K, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "mixed" else "f64", "data": "synthetic",
        "precision": args.precision,
        "config": bench_config(args, cfg, world),
        "e2e": {"value": round(e2e_val, 2), "unit": "MLUPS",
                "h2d_bytes_per_step": up // max(K, 1),
                "d2h_bytes_per_step": n_obj * 10 * 3 * 8,
                "note": f"timed region: lbdem_create from the host tables ({up} B copied once, "
                        f"shown amortised over the {K} steps; the lattice is initialised on "
                        f"the device from the configuration), then every step lbdem_cycle(1) "
                        f"and a read-back of the impactor record to host memory"},
        "roofline": {"bound": "hbm", "achieved": kr["achieved"], "peak": kr["peak"],
                     "unit": "GB/s", "frac": kr["frac"], "traffic": traffic,
                     "peak_kind": kr["peak_kind"],
                     "kernel": "lbStep (fused reconstruct/collide/stream)",
                     "bytes_per_active_node": kr["bytes_per_active_node"],
                     "kernel_ms_per_launch": kr["kernel_ms_per_launch"]},
        "clocks": clk,
        "gpu_launches": int(timed.kernel_launches),
    }
    if extra and not args.no_late and args.precision == "mixed":
        line["late"] = late_window(args, cfg, local, torch)
    if extra and not args.no_fp64:
        line["fp64"] = fp64_form(args, cfg, local, torch)
    line["cpu_baseline"] = None if (not extra or args.no_cpu_baseline) else \
        cpu_baseline(cfg, args.workload, steps=K, budget_s=60.0, single_s=25.0)
    line["serving"] = None if (args.no_serving or not extra) else serving(args)
    line["accuracy"] = None if (args.no_accuracy or not extra) else accuracy(args, cfg)
    print(json.dumps(line), flush=True)


def accuracy(args, cfg) -> dict:
    """The mixed form against the plain FP64 form on the benchmark workload.

    Both run ``--accuracy-steps`` goCycles side by side. Reported:
    - the impactor trajectory error (largest difference of the vertical
      displacement, relative to the largest FP64 displacement);
    - the maximum penetration fluidHeight + r - y of each form;
    - each form's fluid-mass drift over the run;
    - the particle position RMS difference at the end, absolute (length
      units) and relative to the RMS particle displacement of the FP64 form.
    """
    import lbdem
    import numpy as np
    S, blk = args.accuracy_steps, 25
    runs = {p: lbdem.Solver(cfg, precision=p) for p in (lbdem.MIXED, lbdem.PLAIN_FP64)}
    fill = float(cfg.cfg.fluidHeight)
    r0 = float(cfg.cfg.objects[0].r) if cfg.cfg.n_objects else 0.0
    traj = {p: [] for p in runs}
    mass = {p: [] for p in runs}
    for p, sv in runs.items():
        traj[p].append(float(sv.objects()["o_x0"][0][1]))
        mass[p].append(sv.mass_total())
    xinit = runs[lbdem.PLAIN_FP64].particles()["p_x0"]
    done = 0
    while done < S:
        n = min(blk, S - done)
        for p, sv in runs.items():
            sv.cycle(n)
        for p, sv in runs.items():
            traj[p].append(float(sv.objects()["o_x0"][0][1]))
            mass[p].append(sv.mass_total())
        done += n
    xend = {p: sv.particles()["p_x0"] for p, sv in runs.items()}
    for sv in runs.values():
        sv.close()
    prms = float(np.sqrt(np.mean(np.sum((xend[lbdem.MIXED] - xend[lbdem.PLAIN_FP64]) ** 2,
                                        axis=1)))) if len(xinit) else 0.0
    pdisp = float(np.sqrt(np.mean(np.sum((xend[lbdem.PLAIN_FP64] - xinit) ** 2, axis=1)))) \
        if len(xinit) else 0.0
    ym, yf = np.array(traj[lbdem.MIXED]), np.array(traj[lbdem.PLAIN_FP64])
    dm, df = ym - ym[0], yf - yf[0]
    pen = {p: float(np.max(fill + r0 - np.array(traj[p]))) for p in runs}
    drift = {p: float((mass[p][-1] - mass[p][0]) / mass[p][0]) for p in runs}
    return {
        "steps": S, "reference": "plain FP64 form (GPU), same workload and steps",
        "impactor_traj_rel_err": float(np.max(np.abs(dm - df)) / max(np.max(np.abs(df)), 1e-300)),
        "impactor_displacement_fp64": float(df[-1]),
        "max_penetration": {"mixed": pen[lbdem.MIXED], "fp64": pen[lbdem.PLAIN_FP64]},
        "max_penetration_rel_err": abs(pen[lbdem.MIXED] - pen[lbdem.PLAIN_FP64]) /
                                   max(abs(pen[lbdem.PLAIN_FP64]), 1e-300),
        "mass_drift": {"mixed": drift[lbdem.MIXED], "fp64": drift[lbdem.PLAIN_FP64]},
        "particle_position_rms": prms,
        "particle_position_rms_rel": prms / max(pdisp, 1e-300),
        "particle_displacement_rms_fp64": pdisp,
    }


def serving(args) -> dict:
    """Many impact runs on the GPU at once through the run server.

    Seeded streams of varied runs (lattice sides 48-128, vertical up to 160,
    fluid to 60 %, a compressed bed of volume fraction 0.40-0.55 over 80 % of
    the fluid depth, impactor radius 6-16 falling at 0.005-0.05):
    - batch: ``--serve-jobs`` runs of ``--serve-cycles`` goCycles submitted at
      once (jobs/h, makespan, p50/p99);
    - the same first runs in the plain FP64 form and in the mixed form
      (jobs/h of each);
    - Poisson arrivals at each rate of ``--serve-rates`` (jobs per minute):
      ``--sweep-jobs`` runs of ``--sweep-cycles`` goCycles, the same arrival
      times and runs for the mixed and the plain FP64 form; p50/p99
      completion latency from arrival, jobs/h over the stream;
    - batched: ``--serve-batch-jobs`` runs resident at once under the
      schedule the autotuner picks.
    """
    import random
    import casegen
    import lbdem
    import numpy as np

    def job_set(seed, n, tag):
        rng = np.random.default_rng(seed)
        out = []
        for i in range(n):
            d = os.path.join(CACHE, f"serve{seed}bed", f"j{i:03d}")
            case = casegen.serving_case(rng, f"{tag}{i}")
            if not os.path.exists(os.path.join(d, "parameters.cfg")):
                case.write(d)
            out.append(lbdem.LoadedConfig(os.path.join(d, "parameters.cfg")))
        return out

    cfgs = job_set(args.serve_seed, args.serve_jobs, "j")
    C = args.serve_cycles

    def pct(v, q):
        return float(np.percentile(np.asarray(v), q)) if len(v) else None

    def batch(prec, jobs, cycles=C, **opts):
        srv = lbdem.Server(precision=prec, max_active=len(jobs), slice_cycles=args.serve_slice,
                           **opts)
        t0 = time.perf_counter()
        for c in jobs:
            srv.submit(c, cycles)
        res = srv.drain()
        wall = time.perf_counter() - t0
        err = srv.last_error()
        srv.close()
        bad = [r for r in res if r["status"] != 0]
        if bad:
            raise RuntimeError(f"serving run failed: status {bad[0]['status']}: {err}")
        lat = [r["end_time"] - r["submit_time"] for r in res]
        upd = sum(r["active_node_updates"] for r in res)
        starts = [r["start_time"] for r in res]
        return {"jobs": len(jobs), "jobs_per_hour": round(len(jobs) / wall * 3600.0, 1),
                "makespan_s": round(wall, 3), "coupled_mlups": round(upd / wall / 1e6, 1),
                "p50_s": round(pct(lat, 50), 4), "p99_s": round(pct(lat, 99), 4),
                "admission_span_s": round(max(starts) - min(starts), 4),
                "run_p50_s": round(pct([r["end_time"] - r["start_time"] for r in res], 50), 4)}

    def poisson(prec, jobs, arrivals, cycles, names):
        """One Poisson stream. A job the server ends with an error status
        (a run that diverges: a sphere driven out of the domain) is reported
        with its status, cycles done and the server's message; the latency
        percentiles are over the jobs that completed."""
        srv = lbdem.Server(precision=prec, max_active=len(jobs), slice_cycles=args.serve_slice)
        res, ids, k, t0 = [], {}, 0, time.perf_counter()
        while len(res) < len(jobs):
            now = time.perf_counter() - t0
            while k < len(jobs) and arrivals[k] <= now:
                ids[srv.submit(jobs[k], cycles)] = names[k]
                k += 1
            wait = min(0.01, arrivals[k] - now) if k < len(jobs) else 0.05
            res += srv.poll(max(wait, 0.0))
        wall = time.perf_counter() - t0
        err = srv.last_error()
        srv.close()
        done = [r for r in res if r["status"] == 0]
        bad = [r for r in res if r["status"] != 0]
        lat = [r["end_time"] - r["submit_time"] for r in done]
        span = max(r["end_time"] for r in res) - min(r["submit_time"] for r in res)
        out = {"p50_s": round(pct(lat, 50), 3) if lat else None,
               "p99_s": round(pct(lat, 99), 3) if lat else None,
               "jobs_per_hour": round(len(done) / span * 3600.0, 1),
               "wall_s": round(wall, 2), "completed": len(done)}
        if bad:
            out["failed"] = [{"job": ids.get(r["job_id"]), "status": r["status"],
                              "cycles_done": r["cycles"]} for r in bad]
            out["last_error"] = err
        return out

    batch(lbdem.MIXED, cfgs[:2])  # warm-up (module load, allocator pools)
    mixed = batch(lbdem.MIXED, cfgs)
    sub = cfgs[:args.serve_fp64_jobs]
    mixed_sub = batch(lbdem.MIXED, sub)
    fp64_sub = batch(lbdem.PLAIN_FP64, sub)
    # Poisson sweep: the same runs and arrival times for both forms
    rates = [float(v) for v in args.serve_rates.split(",") if v]
    sweep = []
    for rate in rates:
        r2 = random.Random(int(args.serve_seed * 1000 + rate * 10))
        arrivals, t = [], 0.0
        for _ in range(args.sweep_jobs):
            t += r2.expovariate(rate / 60.0)
            arrivals.append(t)
        pick = [(i + int(rate)) % len(cfgs) for i in range(args.sweep_jobs)]
        jobs = [cfgs[j] for j in pick]
        names = [f"j{j}" for j in pick]
        row = {"rate_per_min": rate, "jobs": args.sweep_jobs, "cycles": args.sweep_cycles,
               "job_names": names}
        row["mixed"] = poisson(lbdem.MIXED, jobs, arrivals, args.sweep_cycles, names)
        row["fp64"] = poisson(lbdem.PLAIN_FP64, jobs, arrivals, args.sweep_cycles, names)
        sweep.append(row)
    for c in cfgs:
        c.close()
    # batched configuration: many runs resident at once, their schedule
    # (runs per shared launch group, lattice chunks per block) picked by the
    # autotuner on a sample of them
    many = job_set(args.serve_seed + 1, args.serve_batch_jobs, "b")
    tb, tc, _ = lbdem.tune_server(many[:8], cycles=40, slice_cycles=args.serve_slice)
    batched = batch(lbdem.MIXED, many, batch_runs=tb, chunks_per_block=tc)
    batched["schedule"] = {"batch_runs": tb, "chunks_per_block": tc,
                           "tuned_on": "the first 8 runs, 40 cycles each"}
    for c in many:
        c.close()
    return {
        "sample": f"seeded runs: lattice sides 48-128, vertical 48-160, fluid to 60 %, a "
                  f"compressed bed of volume fraction 0.40-0.55 over 80 % of the fluid depth, "
                  f"impactor r 6-16, vy 0.005-0.05; {args.serve_slice}-cycle slices",
        "batch_mixed": dict(mixed, cycles=C),
        "same_runs": {"runs": len(sub), "cycles": C, "mixed": mixed_sub, "fp64": fp64_sub,
                      "jobs_per_hour_ratio_mixed_over_fp64":
                          round(mixed_sub["jobs_per_hour"] / fp64_sub["jobs_per_hour"], 2)},
        "poisson_sweep": sweep,
        "batched_mixed": dict(batched, cycles=C),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="c2")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-late", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--late-start", type=int, default=600)
    ap.add_argument("--late-steps", type=int, default=100)
    ap.add_argument("--fp64-steps", type=int, default=30)
    ap.add_argument("--accuracy-steps", type=int, default=300)
    ap.add_argument("--serve-jobs", type=int, default=24)
    ap.add_argument("--serve-fp64-jobs", type=int, default=8)
    ap.add_argument("--serve-cycles", type=int, default=200)
    ap.add_argument("--serve-slice", type=int, default=24)
    ap.add_argument("--serve-seed", type=int, default=3)
    ap.add_argument("--serve-batch-jobs", type=int, default=64)
    ap.add_argument("--serve-rates", default="10,20,50",
                    help="Poisson arrival rates (jobs per minute), comma-separated")
    ap.add_argument("--sweep-jobs", type=int, default=4)
    ap.add_argument("--sweep-cycles", type=int, default=5000)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    os.makedirs(CACHE, exist_ok=True)
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)


if __name__ == "__main__":
    main()
