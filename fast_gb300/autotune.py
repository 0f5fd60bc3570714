"""Slab-depth autotuner for the tau solver sweeps.

A block of a solver sweep marches one x-y column tile through ``depth`` z
planes (plus a halo plane on each side).  Deep slabs re-read fewer halo
planes and amortise a block's start-up and its share of the reductions;
shallow slabs give small volumes enough blocks to fill the GPU.  The best
depth depends on the size of the launch, its precision and its solver, so
the library looks it up per size class: floor(log2(W)), W the launch's
tile-planes (the sum over its right-hand sides of x tiles * y tiles * nz).

This module measures that table on the GPU at hand.  For each tuning case (a
cubic volume and a number of right-hand sides) and each candidate depth it
times two solves of a fixed number of iterations (tolerance far below
reach, so every solve runs its iteration budget) and takes the difference,
so allocation, the stencil-code pass, graph capture and the tau pass
cancel and the per-iteration time remains.  Cases of one class are pooled
(time per voxel-iteration summed over the cases); a class without a case
takes the depth of the nearest measured class.  A solve that stops before
its budget (a diverging FP32 BiCGSTAB) leaves that depth unmeasured.

    python -m fast_gb300.autotune             # measure and print the table
    python -m fast_gb300.autotune --install   # ... and use it in this process
    python -m fast_gb300.autotune --write     # ... and write csrc/slab_table.inc
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import time
from typing import Dict, List, Optional, Sequence, Tuple

from . import _native
from .tau import DiffusionSolverType, Dir, Precision, TortuosityParams, solve_directions

CANDIDATES = (2, 4, 8, 16, 32, 64, 128, 256)
DEVICE_TIMED_S = 2e-3  # iterations longer than this are timed by their kernels' events
NUM_CLASSES = 32
# (edge, right-hand sides): cubes across the sizes the engine serves, plus
# the three-direction launches of the batched and benchmark workloads.
DEFAULT_CASES = ((32, 1), (48, 1), (64, 1), (80, 1), (96, 1), (128, 1), (160, 1), (192, 1), (224, 1),
                 (256, 1), (320, 1), (384, 1), (512, 1), (64, 3), (128, 3), (256, 3))
PRECISIONS = (Precision.F64, Precision.F32, Precision.MIXED)
SOLVERS = (DiffusionSolverType.DSOLVER_BICGSTAB, DiffusionSolverType.DSOLVER_CG)
TABLE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "csrc", "slab_table.inc")


def slab_depth(shape, nrhs: int, precision: Precision, solver: DiffusionSolverType) -> Tuple[int, int]:
    """(depth, size class) the library uses for nrhs right-hand sides of a
    volume of ``shape = (nz, ny, nx)``."""
    nz, ny, nx = shape
    d, c = C.c_int32(), C.c_int32()
    st = _native.lib().fast_tau_slab_depth(nx, ny, nz, nrhs, int(precision), int(solver), C.byref(d), C.byref(c))
    if st != 0:
        raise ValueError(f"fast_tau_slab_depth: {_native.last_error()}")
    return int(d.value), int(c.value)


def set_slab_table(precision: Precision, solver: DiffusionSolverType, depths: Optional[Sequence[int]]) -> None:
    """Install the depths of classes 0..len(depths)-1 (0 = no entry) for one
    precision and solver in this process; None restores the built-in table."""
    if depths is None:
        st = _native.lib().fast_tau_set_slab_table(int(precision), int(solver), None, 0)
    else:
        arr = (C.c_int32 * len(depths))(*[int(v) for v in depths])
        st = _native.lib().fast_tau_set_slab_table(int(precision), int(solver), arr, len(depths))
    if st != 0:
        raise ValueError(f"fast_tau_set_slab_table: {_native.last_error()}")


def rule_depth(shape, nrhs: int, precision: Precision, solver: DiffusionSolverType) -> int:
    """The depth of the block-count rule (the full depth, halved while the
    launch has fewer than 608 blocks): the library's choice with an empty
    table.  Leaves the built-in table installed for this precision and
    solver (a table installed earlier in the process is replaced)."""
    lib = _native.lib()
    zeros = (C.c_int32 * NUM_CLASSES)()
    old = os.environ.pop("FAST_TAU_ZC", None)
    try:
        lib.fast_tau_set_slab_table(int(precision), int(solver), zeros, NUM_CLASSES)
        return slab_depth(shape, nrhs, precision, solver)[0]
    finally:
        lib.fast_tau_set_slab_table(int(precision), int(solver), None, 0)
        if old is not None:
            os.environ["FAST_TAU_ZC"] = old


def _volume(edge: int, seed: int):
    from . import volumes
    return volumes.spheres((edge,) * 3, seed=seed, r_min=3.0, r_max=6.0, solid_fraction=0.5)


def _timed(mask, dirs, prec, solver, iters) -> Tuple[float, bool]:
    p = TortuosityParams(tolerance=1e-30, max_iter=iters, precision=prec)
    t0 = time.perf_counter()
    res = solve_directions(mask, dirs, p, solver)
    dt = time.perf_counter() - t0
    return dt, all(r.iterations >= iters for r in res)


_SETUP_KERNELS = ("code", "init", "init64", "tau")


def _per_iteration_device(mask, dirs, prec, solver, depth, iters, repeats) -> Optional[float]:
    """Seconds per iteration from the library's per-kernel CUDA-event
    profile (the iteration kernels only), for launches whose iterations are
    long enough that the event bracketing of every launch costs nothing
    measurable while the allocation of their state would swamp a wall-clock
    difference."""
    old = os.environ.get("FAST_TAU_ZC")
    os.environ["FAST_TAU_ZC"] = str(depth)
    try:
        p = TortuosityParams(tolerance=1e-30, max_iter=iters, precision=prec, profile=True)
        best = None
        for _ in range(repeats + 1):  # the first solve warms up
            res = solve_directions(mask, dirs, p, solver)
            if not all(r.iterations >= iters for r in res):
                return None
            ks = _native.last_stats()["kernels"]
            v = sum(k["ms"] for name, k in ks.items() if name not in _SETUP_KERNELS) / 1e3 / iters
            best = v if best is None else min(best, v)
        return best
    finally:
        if old is None:
            os.environ.pop("FAST_TAU_ZC", None)
        else:
            os.environ["FAST_TAU_ZC"] = old


def _per_iteration(mask, dirs, prec, solver, depth, base_iters, span, repeats) -> Optional[float]:
    """Seconds per iteration of the launch at this depth (None if a solve
    stopped early)."""
    old = os.environ.get("FAST_TAU_ZC")
    os.environ["FAST_TAU_ZC"] = str(depth)
    try:
        _timed(mask, dirs, prec, solver, base_iters)  # warm-up (pool, graph shapes)
        best = None
        for _ in range(repeats):
            t1, ok1 = _timed(mask, dirs, prec, solver, base_iters)
            t2, ok2 = _timed(mask, dirs, prec, solver, base_iters + span)
            if not (ok1 and ok2):
                return None
            v = (t2 - t1) / span
            best = v if best is None else min(best, v)
        return best
    finally:
        if old is None:
            os.environ.pop("FAST_TAU_ZC", None)
        else:
            os.environ["FAST_TAU_ZC"] = old


def measure(cases: Sequence[Tuple[int, int]] = DEFAULT_CASES, precisions: Sequence[Precision] = PRECISIONS,
            solvers: Sequence[DiffusionSolverType] = SOLVERS, candidates: Sequence[int] = CANDIDATES,
            repeats: int = 2, target_s: float = 0.03, log=None) -> List[dict]:
    """Per-iteration times of every case, precision, solver and candidate
    depth (depths above the volume's planes are skipped).  The iteration
    span of a case is sized so that it runs about target_s seconds.  Where
    an iteration takes more than DEVICE_TIMED_S the time is the kernels'
    own (CUDA events), else the wall-clock difference of two solves."""
    rows = []
    for edge, nrhs in cases:
        mask = _volume(edge, seed=1000 + edge)
        dirs = [Dir.X_POS, Dir.Y_POS, Dir.Z_POS, Dir.X_NEG, Dir.Y_NEG, Dir.Z_NEG][:nrhs]
        for prec in precisions:
            for solver in solvers:
                _, cls = slab_depth(mask.shape, nrhs, prec, solver)
                # size the span from one kernel-timed probe at the current depth
                probe = _per_iteration_device(mask, dirs, prec, solver,
                                              slab_depth(mask.shape, nrhs, prec, solver)[0], 16, 1)
                span = 64 if not probe else int(min(2000, max(16, target_s / probe)))
                device = bool(probe) and probe > DEVICE_TIMED_S
                times = {}
                for d in candidates:
                    if d > edge:
                        continue
                    if device:
                        times[d] = _per_iteration_device(mask, dirs, prec, solver, d, span, repeats)
                    else:
                        times[d] = _per_iteration(mask, dirs, prec, solver, d, 8, span, repeats)
                row = {"edge": edge, "nrhs": nrhs, "precision": prec.name, "solver": int(solver), "class": cls,
                       "voxels": edge ** 3 * nrhs, "span": span, "s_per_iter": times,
                       "timing": "kernel events" if device else "wall-clock difference",
                       "rule_depth": rule_depth(mask.shape, nrhs, prec, solver)}
                rows.append(row)
                if log:
                    log(row)
    return rows


def table_from(rows: Sequence[dict], tolerance: float = 0.02) -> Dict[Tuple[str, int], List[int]]:
    """Depth per class for every (precision, solver) in rows: of the depths
    measured in every case of the class, the one of least pooled time per
    voxel-iteration, unless a depth the block-count
    rule gives the class's cases is within `tolerance` of it (then that
    one: a change needs a gain above the timing noise); nearest measured
    class for the rest."""
    out = {}
    keys = sorted({(r["precision"], r["solver"]) for r in rows})
    for key in keys:
        pooled: Dict[int, Dict[int, float]] = {}
        bad: Dict[int, set] = {}
        rule: Dict[int, set] = {}
        for r in rows:
            if (r["precision"], r["solver"]) != key:
                continue
            if r.get("rule_depth"):
                rule.setdefault(r["class"], set()).add(int(r["rule_depth"]))
            acc = pooled.setdefault(r["class"], {})
            for d, t in r["s_per_iter"].items():
                d = int(d)
                if t is None:
                    bad.setdefault(r["class"], set()).add(d)
                else:
                    acc[d] = acc.get(d, 0.0) + t / r["voxels"]
        best = {}
        for c, acc in pooled.items():
            # only depths measured in every case of the class compare fairly
            cases = [r for r in rows if (r["precision"], r["solver"]) == key and r["class"] == c]
            common = set.intersection(*[{int(d) for d in r["s_per_iter"]} for r in cases])
            ok = {d: t for d, t in acc.items() if d in common and d not in bad.get(c, set())}
            if ok:
                fastest = min(ok, key=ok.get)
                near = [d for d in rule.get(c, ()) if d in ok and ok[d] <= ok[fastest] * (1.0 + tolerance)]
                best[c] = min(near, key=ok.get) if near else fastest
        if not best:
            continue
        measured = sorted(best)
        full = []
        for c in range(NUM_CLASSES):
            near = min(measured, key=lambda m: (abs(m - c), m))
            full.append(best[near])
        out[key] = full
    return out


def install(table: Dict[Tuple[str, int], List[int]]) -> None:
    for (prec, solver), depths in table.items():
        set_slab_table(Precision[prec], DiffusionSolverType(solver), depths)


def render(table: Dict[Tuple[str, int], List[int]], device: str, command: str) -> str:
    lines = [
        "// Slab depth (z planes per block) by size class, for the tau solver sweeps.",
        "// kSlabTable[precision][solver][class]: precision F64, F32, MIXED and solver",
        "// BiCGSTAB, CG in their fast_precision / fast_solver order; class =",
        "// floor(log2(W)), W = the launch's tile-planes (sum over its right-hand",
        "// sides of x tiles * y tiles * nz); 0 = no entry (the block-count rule).",
        f"// Measured on {device} by: {command}",
        "#pragma once",
        f"constexpr int kSlabClasses = {NUM_CLASSES};",
        "constexpr int kSlabTable[3][2][kSlabClasses] = {",
    ]
    for prec in PRECISIONS:
        lines.append(f"    {{  // {prec.name}")
        for solver in SOLVERS:
            depths = table.get((prec.name, int(solver)), [0] * NUM_CLASSES)
            lines.append(f"        {{{', '.join(str(int(v)) for v in depths)}}},  // {solver.name}")
        lines.append("    },")
    lines.append("};")
    return "\n".join(lines) + "\n"


def _device_name() -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "the local GPU"


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--cases", default=None, help="comma list of EDGExNRHS, e.g. 64x1,256x3")
    ap.add_argument("--candidates", default=None, help="comma list of depths")
    ap.add_argument("--precisions", default=None, help="comma list of F64,F32,MIXED")
    ap.add_argument("--solvers", default=None, help="comma list of BICGSTAB,CG")
    ap.add_argument("--repeats", type=int, default=2)
    ap.add_argument("--target-s", type=float, default=0.03, help="seconds of iterations per timed span")
    ap.add_argument("--json", default=None, help="write the raw timings here")
    ap.add_argument("--from-json", default=None,
                    help="build the table from timings written by --json (comma list: a later file's rows "
                         "replace an earlier file's rows of the same case, precision and solver)")
    ap.add_argument("--tolerance", type=float, default=0.02,
                    help="keep the block-count rule's depth when within this fraction of the fastest")
    ap.add_argument("--install", action="store_true", help="use the measured table in this process")
    ap.add_argument("--write", nargs="?", const=TABLE_PATH, default=None, help="write the table header")
    a = ap.parse_args(argv)
    cases = DEFAULT_CASES if not a.cases else [tuple(int(v) for v in c.split("x")) for c in a.cases.split(",")]
    cands = CANDIDATES if not a.candidates else [int(v) for v in a.candidates.split(",")]
    precs = PRECISIONS if not a.precisions else [Precision[v] for v in a.precisions.split(",")]
    solvers = SOLVERS if not a.solvers else [DiffusionSolverType["DSOLVER_" + v] for v in a.solvers.split(",")]
    device = _device_name()
    if a.from_json:
        merged = {}
        for path in a.from_json.split(","):
            with open(path) as f:
                saved = json.load(f)
            device = saved.get("device", device)
            for r in saved["rows"]:
                merged[(r["edge"], r["nrhs"], r["precision"], r["solver"])] = r
        rows = list(merged.values())
        for r in rows:
            if "rule_depth" not in r:
                r["rule_depth"] = rule_depth((r["edge"],) * 3, r["nrhs"], Precision[r["precision"]],
                                             DiffusionSolverType(r["solver"]))
    else:
        rows = measure(cases, precs, solvers, cands, a.repeats, a.target_s,
                       log=lambda r: print(json.dumps(r), flush=True))
    table = table_from(rows, a.tolerance)
    if a.json:
        with open(a.json, "w") as f:
            json.dump({"device": device, "rows": rows, "table": {f"{k[0]}/{k[1]}": v for k, v in table.items()}},
                      f, indent=1)
    for (prec, solver), depths in sorted(table.items()):
        print(prec, DiffusionSolverType(solver).name, depths)
    if a.install:
        install(table)
    if a.write:
        opts = [f"--{k} {v}" for k, v in (("cases", a.cases), ("candidates", a.candidates),
                                           ("precisions", a.precisions), ("solvers", a.solvers)) if v]
        opts += [f"--repeats {a.repeats}"] if a.repeats != 2 else []
        opts += [f"--target-s {a.target_s:g}"] if a.target_s != 0.03 else []
        opts += [f"--tolerance {a.tolerance:g}"] if a.tolerance != 0.02 else []
        cmd = " ".join(["python -m fast_gb300.autotune"] + opts + ["--write"])
        with open(a.write, "w") as f:
            f.write(render(table, device, cmd))
        print("wrote", a.write)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
