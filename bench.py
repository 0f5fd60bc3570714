#!/usr/bin/env python
"""Benchmark of the tortuosity engine on one GB300 (or N replicas).

Workload (one "step"): the 256^3 packed-ellipsoid volume (seed 1, semi-major
axis 12 voxels, aspect 0.35, solid fraction 0.55; pore D = 1, solid D = 1e-3,
arithmetic face mean), tau in the three directions x, y, z solved as three
right-hand sides sharing one phase field, BiCGSTAB, FP32 iterations with FP64
residual replacement, tolerance 1e-7 on the FP64 relative residual (BiCGSTAB
needs 1e-7 to meet |dtau|/tau <= 1e-5 on this volume: at 1e-6 the
reference's own FP64 BiCGSTAB misses it by 2-5x).  Metric: tau solves/s (3
per step); |dtau|/tau against the FP64 tol-1e-10 oracle is reported per
direction.  Inputs are synthetic: the reference's
packer cannot run here, so the engine's seeded generator makes a volume of
the same size, shape parameters and solid fraction.

  value   device-resident mask, CUDA events on the launching stream around
          exactly K steps, max over ranks.
  e2e     the public C ABI with a HOST mask (fast_tau_solve_dirs): host to
          device copy of the mask and device to host copy of the results
          inside the timed region.
  roofline the dominant kernel's algorithmic bytes per launch / its average
          CUDA-event duration from one profiled step of the same workload.
  cpu_baseline  the CPU oracle (a C/OpenMP restatement of the reference's
          --cpu path: stored 7-coefficient system + Eigen-style BiCGSTAB, FP64)
          timed on a bounded sample of the same volume and direction.

``--impl reference`` times that CPU restatement alone (the reference itself
cannot be built here: Eigen and glm are absent) and prints its JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOAD = dict(name="ellipsoids256_xyz_bicgstab_mixed", shape=(256, 256, 256), seed=1, semi_major=12.0,
                aspect=0.35, solid_fraction=0.55, dirs=(0, 2, 4), tol=1e-7, max_iter=10000)

# Compulsory bytes per voxel of each kernel (each stream the kernel touches
# read or written once; neighbour re-reads served on chip).  MIXED BiCGSTAB
# runs two sweeps per iteration: step 1 ("bi1") reads r, v, t, p, e, r0, code
# and writes r, p, v, e (41 B); step 2 ("bi2") reads r, v, r0, code and
# writes t (17 B).  The FP64 residual replacement reads x64, e, p, r, v, r0,
# code and writes x64, t (41 B).  CG: step 1 reads r, p, code, writes p;
# step 2 reads p, x, r, code, writes x, r.
KERNEL_BYTES_PER_VOXEL = {"bi1": 41, "bi2": 17, "replace": 41, "tau": 9, "init64": 12, "code": 2, "cg1": 13,
                          "cg2": 21}
# Algorithmic bytes per voxel-iteration of a whole FP32 BiCGSTAB iteration:
# x, r, p, v read+written (32), r0 read (4), phase read twice (2).
ITER_BYTES_FP32_BICGSTAB = 38


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_golden():
    p = os.path.join(ROOT, "tests", "golden", "workloads.json")
    try:
        with open(p) as f:
            return json.load(f)["workloads"].get("ellipsoids256")
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        first = vis.split(",")[0].strip() if vis else ""
        self.index = int(first) if first.isdigit() else index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return ws, rank, local


def spawn_replicas(n: int, argv) -> int:
    """`bench.py --gpus N` started without a launcher: start N copies of this
    script, one per GPU (RANK = LOCAL_RANK = 0..N-1, gloo rendezvous on
    127.0.0.1), as torchrun would, and return the worst exit code."""
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), LOCAL_WORLD_SIZE=str(n),
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__)] + list(argv), env=env))
    codes = [p.wait() for p in procs]
    return next((c for c in codes if c != 0), 0)


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v: float, ws: int) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_volume(use_oracle_generator: bool = False):
    """The benchmark volume.  The CPU arms take it from the oracle's build of
    the generator (the same source file as libfasttau.so's fast_gen_*), so a
    process that times only the CPU path never loads the CUDA library; its
    SHA-256 is checked against the golden record."""
    w = WORKLOAD
    if use_oracle_generator:
        from oracle import oracle as O
        m = O.gen_ellipsoids(w["shape"], w["seed"], w["semi_major"], w["aspect"], w["solid_fraction"])
        g = load_golden()
        if g:
            import hashlib
            if hashlib.sha256(m.tobytes()).hexdigest() != g["sha256"]:
                raise RuntimeError("the generated benchmark volume does not match its golden SHA-256")
        return m
    from fast_gb300 import volumes
    return volumes.ellipsoids(w["shape"], w["seed"], w["semi_major"], w["aspect"], w["solid_fraction"])


def workload_config():
    """The workload both arms measure (the same dict in both JSON lines)."""
    w = WORKLOAD
    return {"workload": w["name"], "volume": "256^3 ellipsoids seed 1 a=12 aspect 0.35 solid 0.55",
            "solver": "BiCGSTAB, Jacobi", "dirs": "x,y,z", "tol": w["tol"],
            "l2": "working set > 129 MB L2 (GPU ~2.4 GB per step); no flush"}


def cpu_solve(mask, dir_: int):
    """One full solve on the host cores: the oracle's FP64 BiCGSTAB in the
    Eigen recurrence (the reference's --cpu path: stored 7-coefficient system,
    diagonal preconditioner) at the workload's tolerance, timed like the
    reference's tauTime (assembly + solve + tau, TauModule.h:87-99).
    Returns (seconds, result)."""
    from oracle import oracle as O
    O.build()
    t0 = time.perf_counter()
    r = O.get_tortuosity(mask, dir=dir_, solver=O.BICGSTAB, tol=WORKLOAD["tol"], max_iter=WORKLOAD["max_iter"],
                         variant=O.EIGEN)
    return time.perf_counter() - t0, r


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def run_reference(args, ws, rank):
    """--impl reference: the reference's CPU path (restated by the oracle;
    the reference itself cannot be built here) on the same workload, every
    host thread.  Each timed step is one complete solve, the direction
    cycling x, y, z from step to step; warm-up steps run the assembly and
    five iterations (they fault in memory and start the thread pool).  Only
    rank 0 works and prints; other ranks return at once."""
    if rank != 0:
        return
    from oracle import oracle as O
    mask = make_volume(use_oracle_generator=True)
    dirs = list(WORKLOAD["dirs"])
    for _ in range(args.warmup):
        O.get_tortuosity(mask, dir=0, solver=O.BICGSTAB, tol=WORKLOAD["tol"], max_iter=5, variant=O.EIGEN)
    secs, per_dir = [], {}
    for i in range(args.steps):
        d = dirs[i % len(dirs)]
        t, r = cpu_solve(mask, d)
        secs.append(t)
        per_dir.setdefault(str(d), []).append({"seconds": t, "iterations": r["iters"], "status": r["status"],
                                               "tau": r["tau"]})
    total = sum(secs)
    value = args.steps / total
    threads = cpu_threads()
    line = {
        "metric": "tau solves/s", "value": value, "unit": "solves/s", "impl": "reference", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded ellipsoid packing stand-in)", "config": workload_config(),
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": threads, "kind": "port",
                         "sample": f"{args.steps} complete FP64 BiCGSTAB solves (Eigen recurrence, Jacobi, tol "
                                   f"{WORKLOAD['tol']:g}) of the 256^3 volume, one direction per step cycling "
                                   f"x, y, z; assembly + solve + tau timed; no extrapolation"},
        "per_direction": {k: {"mean_seconds": statistics.mean(e["seconds"] for e in v),
                              "iterations": v[0]["iterations"], "tau": v[0]["tau"],
                              "all_converged": all(e["status"] == 0 for e in v)} for k, v in per_dir.items()},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    import fast_gb300 as ft
    from fast_gb300 import _native

    w = WORKLOAD
    mask = make_volume()
    N = mask.size
    dirs = [ft.Dir(d) for d in w["dirs"]]
    params = ft.TortuosityParams(tolerance=w["tol"], max_iter=w["max_iter"], precision=ft.Precision.MIXED)
    d_mask = torch.from_numpy(mask).cuda()
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def step():
        return ft.solve_directions_device(d_mask.data_ptr(), mask.shape, dirs, params, ft.DSOLVER_BICGSTAB,
                                          stream=sptr)

    for _ in range(args.warmup):
        res = step()
    torch.cuda.synchronize()
    ok = all(r.status == ft.Status.OK for r in res)

    # --- timed region: exactly K steps, device-resident inputs
    barrier(ws)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    iters = []
    launches = 0
    with ClockSampler(local) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            res = step()
            launches += _native.last_stats()["launches"]
            iters.append(sum(r.iterations for r in res))
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    ms = e0.elapsed_time(e1)
    ms_max = max_over_ranks(ms, ws)
    solves = len(dirs) * args.steps * ws
    value = solves / (ms_max / 1e3)

    # --- end to end through the public C ABI with a host mask
    barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        res_e2e = ft.solve_directions(mask, dirs, params, ft.DSOLVER_BICGSTAB)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    e2e_value = solves / e2e_s

    # --- one profiled step: per-kernel CUDA-event durations
    pparams = ft.TortuosityParams(tolerance=w["tol"], max_iter=w["max_iter"], precision=ft.Precision.MIXED,
                                  profile=True)
    pres = ft.solve_directions_device(d_mask.data_ptr(), mask.shape, dirs, pparams, ft.DSOLVER_BICGSTAB,
                                      stream=sptr)
    prof = _native.last_stats()
    torch.cuda.synchronize()

    if rank != 0:
        return
    peak, peak_kind = load_peaks()
    total_inner = sum(r.iterations for r in pres)
    kern = prof["kernels"]
    # voxels processed by all launches of a kernel kind
    vox = {"bi1": N * total_inner, "bi2": N * total_inner,
           "replace": N * sum(r.outer_steps for r in pres), "tau": N * len(dirs), "code": N,
           "init64": N * len(dirs)}
    dom = max(kern, key=lambda k: kern[k]["ms"])
    dom_bytes = KERNEL_BYTES_PER_VOXEL.get(dom, 0) * vox.get(dom, 0)
    dom_ms = kern[dom]["ms"]
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else 0.0
    iter_ms = sum(kern.get(k, {"ms": 0})["ms"] for k in ("bi1", "bi2", "replace"))
    iter_gbs = ITER_BYTES_FP32_BICGSTAB * N * total_inner / (iter_ms / 1e3) / 1e9 if iter_ms > 0 else 0.0
    launches_per_step = launches / max(args.steps, 1)

    # accuracy against the FP64 tol-1e-10 oracle
    g = load_golden()
    dtau = None
    if g:
        dtau = {}
        for r in res:
            ref = g["dirs"][str(int(r.dir))]["tau_cg_1e-10"]
            dtau[r.dir.name] = abs(r.tau - ref) / ref

    # the same volume and directions through mixed CG, the fastest form that
    # meets the accuracy target (reported beside the BiCGSTAB headline)
    alt = None
    if not args.no_alt:
        cparams = ft.TortuosityParams(tolerance=1e-6, max_iter=w["max_iter"], precision=ft.Precision.MIXED)
        ft.solve_directions_device(d_mask.data_ptr(), mask.shape, dirs, cparams, ft.DSOLVER_CG, stream=sptr)
        torch.cuda.synchronize()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record(stream)
        for _ in range(args.steps):
            cres = ft.solve_directions_device(d_mask.data_ptr(), mask.shape, dirs, cparams, ft.DSOLVER_CG,
                                              stream=sptr)
        a1.record(stream)
        torch.cuda.synchronize()
        cms = a0.elapsed_time(a1) / args.steps
        alt = {"cg_mixed_tol1e-6": {
            "value": len(dirs) / (cms / 1e3), "unit": "solves/s", "ms_per_step": cms,
            "iterations": [r.iterations for r in cres], "all_converged": all(r.status == ft.Status.OK for r in cres),
            "dtau_rel_vs_fp64_oracle": ({r.dir.name: abs(r.tau - g["dirs"][str(int(r.dir))]["tau_cg_1e-10"])
                                         / g["dirs"][str(int(r.dir))]["tau_cg_1e-10"] for r in cres} if g else None)}}
        # the headline with the opt-in float-float iterate in place of FP64
        fparams = ft.TortuosityParams(tolerance=w["tol"], max_iter=w["max_iter"], precision=ft.Precision.MIXED,
                                      replace_float_float=True)
        ft.solve_directions_device(d_mask.data_ptr(), mask.shape, dirs, fparams, ft.DSOLVER_BICGSTAB, stream=sptr)
        torch.cuda.synchronize()
        a0.record(stream)
        for _ in range(args.steps):
            fres = ft.solve_directions_device(d_mask.data_ptr(), mask.shape, dirs, fparams, ft.DSOLVER_BICGSTAB,
                                              stream=sptr)
        a1.record(stream)
        torch.cuda.synchronize()
        fms = a0.elapsed_time(a1) / args.steps
        alt["bicgstab_mixed_float_float_iterate"] = {
            "value": len(dirs) / (fms / 1e3), "unit": "solves/s", "ms_per_step": fms,
            "iterations": [r.iterations for r in fres], "all_converged": all(r.status == ft.Status.OK for r in fres),
            "dtau_rel_vs_fp64_oracle": ({r.dir.name: abs(r.tau - g["dirs"][str(int(r.dir))]["tau_cg_1e-10"])
                                         / g["dirs"][str(int(r.dir))]["tau_cg_1e-10"] for r in fres} if g else None),
            "dtau_rel_vs_fp64_iterate": {a.dir.name: abs(a.tau - b.tau) / b.tau for a, b in zip(fres, res)}}

    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        secs, r = cpu_solve(mask, 0)
        cpu = {"value": 1.0 / secs, "unit": "solves/s", "cores": cpu_threads(), "kind": "port",
               "sample": f"one complete solve of this volume in x: the oracle's FP64 BiCGSTAB (Eigen recurrence, "
                         f"the reference --cpu path; Jacobi, tol {w['tol']:g}), assembly + solve + tau, "
                         f"{r['iters']} iterations in {secs:.1f} s; no extrapolation",
               "tau": r["tau"], "iterations": r["iters"]}

    line = {
        "metric": "tau solves/s", "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded ellipsoid packing stand-in)",
        "config": workload_config(),
        "precision": "FP32 iterations + FP64 residual replacement", "parallelism": f"replicas x{ws}",
        "rhs": "x, y, z as 3 right-hand sides of one launch sharing the phase field",
        "voxel_iters_per_s": N * (sum(iters) / len(iters)) * ws / (ms_max / 1e3 / args.steps),
        "iterations_per_step": sum(iters) / len(iters),
        "all_converged": ok,
        "dtau_rel_vs_fp64_oracle": dtau,
        "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": int(N),
                "d2h_bytes_per_step": int(len(dirs) * C_RESULT_BYTES)},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": dom_bytes / max(kern[dom]["launches"], 1),
                     "avg_launch_ms": dom_ms / max(kern[dom]["launches"], 1),
                     "traffic": NCU_TRAFFIC.get(dom),
                     "iteration_gbs_at_38B": iter_gbs, "iteration_frac_at_38B": iter_gbs / peak},
        "kernel_profile_ms": {k: round(v["ms"], 3) for k, v in kern.items()},
        "gpu_launches": int(launches),
        "gpu_launches_per_step": launches_per_step,
        "clocks": clk.summary(),
    }
    if alt:
        line["alternatives"] = alt
    if cpu:
        line["cpu_baseline"] = cpu
    if ws == 1 and not args.no_subrecords:
        # the two other targets of the specification, measured in the same
        # run: the 1024^3 PCG iteration against the HBM roofline, and the
        # serving stream against the plain drop-in solver (a bounded sample of
        # the 10,000-request stream: the first --c4-requests of its requests)
        del d_mask
        torch.cuda.empty_cache()
        line["c5"] = c5_record(args.c5_edge)
        line["c4"] = c4_record(args.c4_requests, args.c4_rates, args.c4_plain_sample)
    print(json.dumps(line), flush=True)


C_RESULT_BYTES = 40  # sizeof(fast_tau_result)
# DRAM bytes (read + write) per bench launch of each kernel, from one ncu
# --set full capture of a one-direction launch of the same volume
# (profiles/), scaled by 3 to the three right-hand sides a bench launch
# processes (traffic grows with the voxels).
NCU_TRAFFIC = {"bi1": 3 * 672.3e6, "bi2": 3 * 276.2e6}
# DRAM bytes per voxel-iteration of the two PCG sweeps at the large-volume
# slab depth (ncu dram__bytes_read.sum + dram__bytes_write.sum of OpCG1 and
# OpCG2 on the 512^3 spheres at 256 planes per block: 13.04 + 21.48).
C5_DRAM_BYTES_PER_VOXEL_ITER = 34.52


# ---------------------------------------------------------------------------
# Other configurations of the workload table (each prints its own JSON line)
# ---------------------------------------------------------------------------
def _line(metric, value, unit, args, ms_per_step, dtype, config, **extra):
    d = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
         "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
         "dtype": dtype, "data": "synthetic (seeded generator stand-ins)", "config": config}
    d.update(extra)
    return d


def _events(stream):
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def run_c1(args):
    """Plain drop-in: 64^3 spheres (seed 0, r = 5, solid 0.60), direction x,
    Jacobi-PCG, tol 1e-6, FP64, through fast_tau_solve with a host mask (the
    getTortuosity<double> replacement), one solve per step; tau compared with
    the oracle's Eigen CG (the reference --cpu path) on the same volume."""
    import torch
    import fast_gb300 as ft
    from fast_gb300 import volumes
    from oracle import oracle as O
    m = volumes.spheres((64, 64, 64), seed=0, r_min=5.0, solid_fraction=0.60)
    p = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-6, max_iter=10000, precision=ft.Precision.F64)
    for _ in range(args.warmup):
        ft.get_tortuosity(m, p, ft.DSOLVER_CG)
    lat = []
    it = [0]
    for _ in range(args.steps):
        t0 = time.perf_counter()
        tau = ft.get_tortuosity(m, p, ft.DSOLVER_CG, iterations_out=it)
        lat.append(time.perf_counter() - t0)
    O.build()
    t0 = time.perf_counter()
    ref = O.get_tortuosity(m, dir=0, solver=O.CG, tol=1e-6, max_iter=10000, variant=O.EIGEN)
    t_cpu = time.perf_counter() - t0
    w = json.load(open(os.path.join(ROOT, "tests", "golden", "workloads.json")))["workloads"]["spheres64"]
    exact = w["dirs"]["0"]["tau_cg_1e-10"]
    mean = statistics.mean(lat)
    line = _line("tau solves/s", 1.0 / mean, "solves/s", args, mean * 1e3, "f64",
                 {"workload": "c1_spheres64_x_cg_f64_dropin", "volume": "64^3 spheres seed 0 r=5 solid 0.60",
                  "solver": "Jacobi-PCG", "tol": 1e-6, "api": "fast_tau_solve (host mask, synchronous)"},
                 tau=tau, iterations=it[0], latency_ms={"p50": 1e3 * statistics.median(lat), "max": 1e3 * max(lat)},
                 tau_cpu_eigen=ref["tau"], iterations_cpu_eigen=ref["iters"],
                 dtau_rel_vs_cpu_eigen=abs(tau - ref["tau"]) / ref["tau"],
                 dtau_rel_vs_fp64_oracle_1e10=abs(tau - exact) / exact,
                 cpu_baseline={"value": 1.0 / t_cpu, "unit": "solves/s", "cores": os.cpu_count() or 1,
                               "kind": "port", "sample": "oracle FP64 Eigen-recurrence CG, full solve of the same "
                                                         "volume (assembly + solve + tau)"},
                 e2e={"value": 1.0 / mean, "unit": "solves/s", "h2d_bytes_per_step": int(m.size),
                      "d2h_bytes_per_step": 40})
    print(json.dumps(line), flush=True)


def c3_volumes():
    """64 volumes, seeds 100-163: each dimension uniform in 64..192, sphere
    radius uniform 3..8 voxels, solid fraction uniform 0.40..0.75, direction
    uniform over x, y, z."""
    from concurrent.futures import ThreadPoolExecutor
    from fast_gb300 import volumes
    specs = []
    for seed in range(100, 164):
        rng = np.random.default_rng(seed)
        shape = tuple(int(v) for v in rng.integers(64, 193, size=3))
        frac = float(rng.uniform(0.40, 0.75))
        d = int(rng.choice([0, 2, 4]))
        specs.append((shape, seed, frac, d))
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        masks = list(ex.map(lambda s: volumes.spheres(s[0], seed=s[1], r_min=3.0, r_max=8.0, solid_fraction=s[2]),
                            specs))
    return [(m, s[3]) for m, s in zip(masks, specs)]


def run_c3(args):
    """Batched launch: the 64 uneven volumes of c3_volumes() solved together
    (fast_tau_solve_batch_device, MIXED PCG, tol 1e-6), against the plain
    drop-in solver (FP64, one volume per call) and MIXED one per call on the
    same volumes; |dtau|/tau against FP64 PCG at tol 1e-10 (batched)."""
    import torch
    import fast_gb300 as ft
    from fast_gb300 import _native
    vols = c3_volumes()
    d_masks = [torch.from_numpy(m).cuda() for m, _ in vols]
    spec = [(t.data_ptr(), m.shape, d) for t, (m, d) in zip(d_masks, vols)]
    stream = torch.cuda.current_stream()
    p = ft.TortuosityParams(tolerance=1e-6, max_iter=10000, precision=ft.Precision.MIXED)
    for _ in range(args.warmup):
        res = ft.solve_batch_device(spec, p, ft.DSOLVER_CG, stream=stream.cuda_stream)
    torch.cuda.synchronize()
    e0, e1 = _events(stream)
    launches = 0
    e0.record(stream)
    for _ in range(args.steps):
        res = ft.solve_batch_device(spec, p, ft.DSOLVER_CG, stream=stream.cuda_stream)
        launches += _native.last_stats()["launches"]
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    value = len(vols) / (ms / 1e3)

    def one_at_a_time(prec, n):
        q = ft.TortuosityParams(tolerance=1e-6, max_iter=10000, precision=prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for (ptr, shape, d) in spec[:n]:
            ft.solve_directions_device(ptr, shape, [ft.Dir(d)], q, ft.DSOLVER_CG, stream=stream.cuda_stream)
        torch.cuda.synchronize()
        return n / (time.perf_counter() - t0)

    plain_f64 = one_at_a_time(ft.Precision.F64, len(vols))
    plain_mixed = one_at_a_time(ft.Precision.MIXED, len(vols))
    ref = ft.solve_batch_device(spec, ft.TortuosityParams(tolerance=1e-10, max_iter=100000,
                                                          precision=ft.Precision.F64), ft.DSOLVER_CG,
                                stream=stream.cuda_stream)
    dt = [abs(a.tau - b.tau) / b.tau for a, b in zip(res, ref)]
    voxels = sum(m.size for m, _ in vols)
    line = _line("tau solves/s", value, "solves/s", args, ms, "f32+f64",
                 {"workload": "c3_batch64_uneven_cg_mixed", "volumes": "64, seeds 100-163, dims U[64,192], "
                  "sphere r U[3,8], solid U[0.40,0.75], dir U{x,y,z}", "solver": "Jacobi-PCG", "tol": 1e-6,
                  "api": "fast_tau_solve_batch_device (one launch per solver step over all volumes, "
                         "16-iteration CUDA graphs)"},
                 voxels=int(voxels), all_converged=all(r.status == ft.Status.OK for r in res),
                 iterations={"min": min(r.iterations for r in res), "max": max(r.iterations for r in res)},
                 plain_dropin_f64_solves_per_s=plain_f64, plain_mixed_solves_per_s=plain_mixed,
                 speedup_vs_plain_f64=value / plain_f64, speedup_vs_plain_mixed=value / plain_mixed,
                 dtau_rel_vs_fp64_1e10={"max": max(dt), "median": statistics.median(dt)},
                 gpu_launches_per_step=launches / max(args.steps, 1))
    print(json.dumps(line), flush=True)


def c4_requests(n, seed=2024, pool=0):
    """Serving stream requests: edge log-uniform in [32, 384] (cubic),
    spheres (r U[3,8]) or ellipsoids (semi-major 8, aspect U[0.1,1.0]),
    solid fraction U[0.40,0.75], direction uniform over the six, CG or
    BiCGSTAB.  With pool > 0 only the first `pool` volumes are generated and
    request k carries volume k % pool (with its own direction and solver), so
    a long stream fits in host memory; the size mix is the pool's."""
    from concurrent.futures import ThreadPoolExecutor
    from fast_gb300 import volumes
    rng = np.random.default_rng(seed)
    specs = []
    for k in range(n):
        e = int(round(float(np.exp(rng.uniform(np.log(32), np.log(384))))))
        frac = float(rng.uniform(0.40, 0.75))
        kind = "spheres" if rng.random() < 0.5 else "ellipsoids"
        aspect = float(rng.uniform(0.1, 1.0))
        specs.append(dict(edge=e, frac=frac, kind=kind, aspect=aspect, seed=int(rng.integers(1 << 30)),
                          dir=int(rng.integers(6)), solver=int(rng.integers(2))))
    npool = n if pool <= 0 or pool >= n else pool
    for k in range(npool, n):  # volume of request k: the pool's entry k % npool
        src = specs[k % npool]
        specs[k].update(edge=src["edge"], frac=src["frac"], kind=src["kind"], aspect=src["aspect"],
                        seed=src["seed"])

    def gen(sp):
        sh = (sp["edge"],) * 3
        if sp["kind"] == "spheres":
            return volumes.spheres(sh, seed=sp["seed"], r_min=3.0, r_max=8.0, solid_fraction=sp["frac"])
        return volumes.ellipsoids(sh, sp["seed"], 8.0, sp["aspect"], sp["frac"])
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        vols = list(ex.map(gen, specs[:npool]))
    masks = [vols[k % npool] for k in range(n)]
    return specs, masks


def c4_record(n_requests, rates, plain_sample, chunk=16, pool=0, max_pending=256, progress=False):
    """Serving stream: Poisson arrivals of c4_requests(n_requests) at each
    rate into one TauServer (MIXED, tol 1e-6); latency = completion minus
    arrival; against the plain drop-in solver (FP64, one request per call,
    back to back) on the same requests (all, or `plain_sample` of them evenly
    spaced through the stream so the sample keeps its size mix).  Requests
    that have arrived wait on the client side (their buffers uncopied) while
    `max_pending` submitted requests are still queued in the server, so an
    overloaded stream does not hold a host copy of every waiting volume;
    their latency still counts from their arrival."""
    import torch
    import fast_gb300 as ft
    from fast_gb300.serve import TauServer
    t0g = time.perf_counter()
    specs, masks = c4_requests(n_requests, pool=pool)
    t_gen = time.perf_counter() - t0g
    out = {}
    rng = np.random.default_rng(7)
    for rate in rates:
        gaps = rng.exponential(1.0 / rate, size=len(masks))
        arrivals = np.cumsum(gaps)
        with TauServer(tolerance=1e-6, chunk=chunk) as srv:
            t0 = srv.now()
            k = 0
            done = []
            while k < len(masks) or srv.busy():
                now = srv.now() - t0
                room = max_pending - srv.stats()["pending"] if max_pending > 0 else len(masks)
                while k < len(masks) and arrivals[k] <= now and room > 0:
                    srv.submit(masks[k], ft.Dir(specs[k]["dir"]), ft.DiffusionSolverType(specs[k]["solver"]))
                    k += 1
                    room -= 1
                if srv.busy():
                    done.extend(srv.poll())
                elif k < len(masks):
                    time.sleep(max(0.0, min(0.01, arrivals[k] - (srv.now() - t0))))
            span = max(c.t_done for c in done) - (t0 + arrivals[0])
        by_ticket = sorted(done, key=lambda c: c.ticket)
        lat = [c.t_done - (t0 + arrivals[i]) for i, c in enumerate(by_ticket)]
        out[str(int(rate))] = {"solves_per_s": len(done) / span, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                               "p99_ms": 1e3 * float(np.percentile(lat, 99)),
                               "arrival_span_s": float(arrivals[-1] - arrivals[0]), "makespan_s": span,
                               "all_converged": all(c.result.status == ft.Status.OK for c in done)}
        if progress:
            r_ = out[str(int(rate))]
            print(f"c4 rate {rate:g}/s: {r_['solves_per_s']:.2f} solves/s, p50 {r_['p50_ms'] / 1e3:.1f} s, "
                  f"p99 {r_['p99_ms'] / 1e3:.1f} s", file=sys.stderr, flush=True)
    n = len(masks)
    picks = list(range(n)) if plain_sample <= 0 or plain_sample >= n else \
        sorted({int(i) for i in np.linspace(0, n - 1, plain_sample)})
    q = {s_: ft.TortuosityParams(tolerance=1e-6, precision=ft.Precision.F64) for s_ in (0, 1)}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in picks:
        ft.solve_directions(masks[k], [ft.Dir(specs[k]["dir"])], q[specs[k]["solver"]],
                            ft.DiffusionSolverType(specs[k]["solver"]))
    plain = len(picks) / (time.perf_counter() - t0)
    best = max(v["solves_per_s"] for v in out.values())
    voxels = [m.size for m in masks]
    return {"requests": n, "distinct_volumes": (pool if 0 < pool < n else n), "rates": out,
            "best_solves_per_s": best,
            "plain_dropin_f64_solves_per_s": plain, "plain_sample": len(picks),
            "speedup_vs_plain_f64": best / plain,
            "voxels_per_request": {"mean": float(np.mean(voxels)), "max": int(max(voxels)),
                                   "plain_sample_mean": float(np.mean([voxels[k] for k in picks]))},
            "generation_seconds": t_gen,
            "mix": "edge log-U[32,384] cubic, spheres r U[3,8] or ellipsoids aspect U[0.1,1], "
                   "solid U[0.40,0.75], dir U(6), CG or BiCGSTAB",
            "server": "TauServer MIXED tol 1e-6, 16-iteration chunks, admission by HBM footprint",
            "client_queue": f"arrived requests wait uncopied while {max_pending} are queued in the server"}


def run_c4(args):
    import fast_gb300  # noqa: F401
    rec = c4_record(args.requests, args.rates, args.plain_sample, pool=args.c4_pool, progress=True)
    best = rec["best_solves_per_s"]
    line = _line("tau solves/s", best, "solves/s", args, 1e3 / best, "f32+f64",
                 {"workload": "c4_serving_stream", "requests": rec["requests"], "mix": rec["mix"], "tol": 1e-6,
                  "server": rec["server"]}, **{k: v for k, v in rec.items() if k not in ("mix", "server")})
    print(json.dumps(line), flush=True)


def c5_record(edge=1024, reference=False):
    """Large volume: edge^3 spheres (seed 7, r = 10, solid 0.65); GPU CCL of
    the pore phase (label count against the oracle's, components spanning
    x, canonical order checked on the device), then MIXED Jacobi-PCG in x to
    tol 1e-6, timed with CUDA events, and once more with every kernel timed:
    the iteration kernels' algorithmic GB/s (25 B per voxel-iteration)
    against the measured HBM peak, and tau against the FP64 tau of the golden
    record (GPU FP64 PCG, tol 1e-10)."""
    import torch
    import fast_gb300 as ft
    from fast_gb300 import _native, ccl, volumes
    n = edge
    t0 = time.perf_counter()
    m = volumes.spheres((n, n, n), seed=7, r_min=10.0, solid_fraction=0.65)
    t_gen = time.perf_counter() - t0
    d_mask = torch.from_numpy(m).cuda()
    del m
    stream = torch.cuda.current_stream()
    d_labels = torch.empty((n, n, n), dtype=torch.int32, device="cuda")
    ccl.get_volume_ccl_device(d_mask.data_ptr(), (n, n, n), d_labels.data_ptr(), background=255, boundary=False)
    torch.cuda.synchronize()
    e0, e1 = _events(stream)
    e0.record(stream)
    c = ccl.get_volume_ccl_device(d_mask.data_ptr(), (n, n, n), d_labels.data_ptr(), background=255)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_ccl = e0.elapsed_time(e1)
    lab = d_labels.view(-1)
    fg = lab != 0
    first = torch.full((c.num_labels,), lab.numel(), dtype=torch.int64, device="cuda")
    idx = torch.nonzero(fg).squeeze(1)
    first.scatter_reduce_(0, lab[idx].long(), idx, reduce="amin")
    canonical = bool((first[2:] > first[1:-1]).all().item()) if c.num_labels > 2 else True
    spanning = c.get_dir_mask(ft.Dir.X_NEG, ft.Dir.X_POS)
    pores = int(fg.sum().item())
    sizes = torch.bincount(lab.long(), minlength=c.num_labels)
    span_vox = int(sizes[torch.from_numpy(spanning.astype(bool)).cuda()].sum().item())
    del first, idx, fg, sizes, lab, d_labels
    torch.cuda.empty_cache()
    golden = None
    try:
        with open(os.path.join(ROOT, "tests", "golden", "workloads.json")) as f:
            golden = json.load(f)["workloads"].get(f"spheres{n}")
    except Exception:
        golden = None

    p = ft.TortuosityParams(tolerance=1e-6, max_iter=100000, precision=ft.Precision.MIXED)
    e0.record(stream)
    res = ft.solve_directions_device(d_mask.data_ptr(), (n, n, n), [ft.Dir.X_POS], p, ft.DSOLVER_CG,
                                     stream=stream.cuda_stream)[0]
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    pp = ft.TortuosityParams(tolerance=1e-6, max_iter=100000, precision=ft.Precision.MIXED, profile=True)
    ft.solve_directions_device(d_mask.data_ptr(), (n, n, n), [ft.Dir.X_POS], pp, ft.DSOLVER_CG,
                               stream=stream.cuda_stream)
    prof = _native.last_stats()["kernels"]
    N = n ** 3
    iter_ms = sum(prof.get(k, {"ms": 0})["ms"] for k in ("cg1", "cg2", "replace"))
    gbs = 25.0 * N * res.iterations / (iter_ms / 1e3) / 1e9
    sweep_ms = sum(prof.get(k, {"ms": 0})["ms"] for k in ("cg1", "cg2"))
    dram_gbs = C5_DRAM_BYTES_PER_VOXEL_ITER * N * res.iterations / (sweep_ms / 1e3) / 1e9
    per_kernel = {}
    for k, b in (("cg1", 13), ("cg2", 21)):
        if k in prof and prof[k]["ms"] > 0:
            per_kernel[k] = {"bytes_per_voxel": b, "ms_per_launch": prof[k]["ms"] / max(prof[k]["launches"], 1),
                             "gbs": b * N * res.iterations / (prof[k]["ms"] / 1e3) / 1e9}
    peak, kind = load_peaks()
    rec = {"volume": f"{n}^3 spheres seed 7 r=10 solid 0.65", "solver": "MIXED Jacobi-PCG, x, tol 1e-6",
           "solve_ms": ms, "solves_per_s": 1e3 / ms, "tau": res.tau, "iterations": res.iterations,
           "status": int(res.status), "outer_steps": res.outer_steps,
           "stencil_iteration": {"gbs_at_25B": gbs, "peak": peak, "peak_kind": kind, "frac": gbs / peak,
                                 "frac_of_8000": gbs / 8000.0, "iteration_ms": iter_ms / max(res.iterations, 1),
                                 "dram_gbs": dram_gbs, "dram_frac": dram_gbs / peak,
                                 "dram_bytes_per_voxel_iter": C5_DRAM_BYTES_PER_VOXEL_ITER,
                                 "kernels": per_kernel,
                                 "kernel_ms": {k: round(v["ms"], 2) for k, v in prof.items()}},
           "ccl": {"ms": ms_ccl, "num_labels": c.num_labels, "canonical_order": canonical, "pore_voxels": pores,
                   "x_spanning_components": int(spanning[1:].sum()),
                   "x_spanning_pore_fraction": span_vox / max(pores, 1),
                   "num_labels_equals_oracle": (c.num_labels == golden["ccl"]["num_labels"]) if golden else None},
           "generation_seconds": t_gen}
    if golden and "0" in golden.get("dirs", {}):
        ref = golden["dirs"]["0"]["tau_cg_1e-10"]
        rec["tau_fp64_1e-10"] = ref
        rec["dtau_rel_vs_fp64"] = abs(res.tau - ref) / ref
        rec["fp64_reference"] = golden["dirs"]["0"].get("solver_cg_1e-10")
    if reference:
        q = ft.TortuosityParams(tolerance=1e-9, max_iter=200000, precision=ft.Precision.MIXED)
        r9 = ft.solve_directions_device(d_mask.data_ptr(), (n, n, n), [ft.Dir.X_POS], q, ft.DSOLVER_CG,
                                        stream=stream.cuda_stream)[0]
        rec["tau_mixed_1e-9"] = r9.tau
        rec["dtau_rel_vs_mixed_1e-9"] = abs(res.tau - r9.tau) / r9.tau
    del d_mask
    torch.cuda.empty_cache()
    return rec


def run_c5(args):
    rec = c5_record(args.c5_edge, reference=not args.c5_no_reference)
    line = _line("tau solves/s", rec["solves_per_s"], "solves/s", args, rec["solve_ms"], "f32+f64",
                 {"workload": f"c5_spheres{args.c5_edge}_x_cg_mixed", "volume": rec["volume"],
                  "solver": "Jacobi-PCG", "tol": 1e-6}, **rec)
    print(json.dumps(line), flush=True)


def run_alpha(args):
    """Reactive area (`fast alpha`) on the large volume: 1024^3 spheres (seed
    7, r = 10, solid 0.65), device-resident.  Timed (CUDA events, after
    warm-up): the labelling of the pore phase alone, the full tensor call
    (labelling + one seven-field marching-cubes pass), and the one-field
    area pass.  The one-field pass reads 1 B per voxel (the mask); the
    seven-field pass reads 5 B per voxel (mask + 32-bit label; the per-label
    face bits stay in L2).  CPU baseline: the oracle's area of the same field
    on a bounded 256^3 corner of the volume, all host threads."""
    import ctypes as C
    import torch
    from fast_gb300 import _native, alpha, ccl, volumes
    from oracle import oracle as O
    n = args.c5_edge
    m = volumes.spheres((n, n, n), seed=7, r_min=10.0, solid_fraction=0.65)
    sample = np.ascontiguousarray(m[:256, :256, :256]) if not args.no_cpu_baseline else None
    d_mask = torch.from_numpy(m).cuda()
    del m
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    N = n ** 3
    d_labels = torch.empty((n, n, n), dtype=torch.int32, device="cuda")

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        e0, e1 = _events(stream)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / args.steps

    ms_ccl = timed(lambda: ccl.get_volume_ccl_device(d_mask.data_ptr(), (n, n, n), d_labels.data_ptr(),
                                                     background=255))
    del d_labels
    torch.cuda.empty_cache()
    out = {}

    def tensor():
        out["t"] = alpha.get_reactive_area_density_tensor_device(d_mask.data_ptr(), (n, n, n), 0.5, sp)

    ms_tensor = timed(tensor)
    one = C.c_double()
    L = _native.lib()

    def area1():
        L.fast_reactive_area_device(C.c_void_p(d_mask.data_ptr()), n, n, n, 0.5, C.byref(one), C.c_void_p(sp))

    ms_area1 = timed(area1)
    t, solid = out["t"]
    peak, kind = load_peaks()
    ms_area7 = max(ms_tensor - ms_ccl, 1e-9)
    cpu = None
    if sample is not None:
        import multiprocessing
        t0 = time.perf_counter()
        a_cpu = O.reactive_area(sample)
        dt = time.perf_counter() - t0
        cpu = {"value": sample.size / dt, "unit": "voxels/s", "cores": multiprocessing.cpu_count(), "kind": "port",
               "sample": "oracle area of the solid field on the 256^3 corner of the volume", "area": a_cpu}
    line = _line("reactive area voxels/s", N / (ms_tensor / 1e3), "voxels/s", args, ms_tensor, "u8+u32->f32/f64",
                 {"workload": f"alpha_spheres{n}_tensor", "volume": f"{n}^3 spheres seed 7 r=10 solid 0.65",
                  "isovalue": 0.5, "inputs": "device-resident, larger than L2"},
                 tensor=t, area_solid=solid, area_one_field=one.value,
                 ms={"labelling": ms_ccl, "tensor_total": ms_tensor, "area_pass_7_fields": ms_area7,
                     "area_pass_1_field": ms_area1},
                 roofline={"bound": "hbm", "kernel": "alpha_kernel<false>", "achieved": N / (ms_area1 / 1e3) / 1e9,
                           "peak": peak, "unit": "GB/s", "frac": N / (ms_area1 / 1e3) / 1e9 / peak,
                           "peak_kind": kind, "bytes_per_voxel": 1,
                           "seven_field_gbs_at_5B": 5 * N / (ms_area7 / 1e3) / 1e9},
                 cpu_baseline=cpu)
    print(json.dumps(line), flush=True)


def run_ncu_case(args):
    """A short, fixed run of the workload's kernels for profiler captures:
    the bench volume (the 64^3 plain drop-in volume with --workload c1, the
    large-volume spheres at --c5-edge with --workload c5),
    one direction (x), BiCGSTAB (or CG with --ncu-solver cg) in MIXED (FP64
    for c1, or --ncu-precision) stopped after --ncu-iters iterations.
    Prints the iteration count; times nothing."""
    import torch
    import fast_gb300 as ft
    from fast_gb300 import volumes
    if args.workload == "c1":
        name = "c1_spheres64"
        mask = volumes.spheres((64, 64, 64), seed=0, r_min=5.0, solid_fraction=0.60)
        prec = args.ncu_precision or "f64"
    elif args.workload == "c5":
        n = args.c5_edge
        name = f"c5_spheres{n}"
        mask = volumes.spheres((n, n, n), seed=7, r_min=10.0, solid_fraction=0.65)
        prec = args.ncu_precision or "mixed"
    else:
        name = WORKLOAD["name"]
        mask = make_volume()
        prec = args.ncu_precision or "mixed"
    d_mask = torch.from_numpy(mask).cuda()
    p = ft.TortuosityParams(tolerance=1e-12, max_iter=args.ncu_iters, precision=ft.Precision[prec.upper()])
    solver = ft.DSOLVER_CG if args.ncu_solver == "cg" else ft.DSOLVER_BICGSTAB
    res = ft.solve_directions_device(d_mask.data_ptr(), mask.shape, [ft.Dir.X_POS], p, solver)
    torch.cuda.synchronize()
    print(json.dumps({"ncu_case": name + "_x", "precision": prec, "iterations": res[0].iterations,
                      "status": int(res[0].status)}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-alt", action="store_true", help="skip the mixed-CG comparison measurement")
    ap.add_argument("--ncu-case", action="store_true",
                    help="run a short fixed slice of the workload for profiler captures and exit")
    ap.add_argument("--ncu-iters", type=int, default=12)
    ap.add_argument("--ncu-solver", default="bicgstab", choices=["bicgstab", "cg"])
    ap.add_argument("--ncu-precision", default=None, choices=["f64", "f32", "mixed"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5", "alpha"],
                    help="c2 (default) is the headline; the others print their own line")
    ap.add_argument("--requests", type=int, default=10000, help="c4: requests in the stream")
    ap.add_argument("--rates", type=float, nargs="+", default=[50.0, 200.0, 1000.0, 2000.0],
                    help="c4: arrival rates (1/s)")
    ap.add_argument("--plain-sample", type=int, default=200,
                    help="c4: requests timed on the plain solver, evenly spaced (0: all of them)")
    ap.add_argument("--c5-edge", type=int, default=1024)
    ap.add_argument("--c5-no-reference", action="store_true")
    ap.add_argument("--no-subrecords", action="store_true",
                    help="headline only: skip the large-volume (c5) and serving (c4) records of the default line")
    ap.add_argument("--c4-requests", type=int, default=200, help="requests of the serving record in the default line")
    ap.add_argument("--c4-rates", type=float, nargs="+", default=[10.0, 50.0, 200.0, 1000.0, 2000.0],
                    help="serving record of the default line: arrival rates (1/s); 10/s is below saturation")
    ap.add_argument("--c4-plain-sample", type=int, default=24)
    ap.add_argument("--c4-pool", type=int, default=500,
                    help="c4: distinct volumes generated for the stream (request k uses volume k %% pool)")
    ap.add_argument("--replica-check", action="store_true",
                    help="start the ranks, meet in a barrier and a max over ranks, print them and exit")
    args = ap.parse_args()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(spawn_replicas(args.gpus, sys.argv[1:]))
    if args.replica_check:
        ws, rank, local = dist_init()
        barrier(ws)
        m = max_over_ranks(1.5 + rank, ws)
        if rank == 0:
            print(json.dumps({"replica_check": True, "world_size": ws, "max_over_ranks": m}), flush=True)
        barrier(ws)
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    if args.ncu_case:
        from fast_gb300 import build
        build.build()
        run_ncu_case(args)
        return
    if args.workload != "c2":
        from fast_gb300 import build
        build.build()
        import torch
        torch.cuda.set_device(0)
        {"c1": run_c1, "c3": run_c3, "c4": run_c4, "c5": run_c5, "alpha": run_alpha}[args.workload](args)
        return
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    else:
        from fast_gb300 import build
        build.build()
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
