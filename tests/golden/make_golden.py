"""Generates the golden fixtures in this folder from the CPU oracle.

The reference ships no tests, golden vectors or sample data, and it cannot be
built here (Eigen and glm are absent), so its outputs cannot be recorded.
These fixtures instead pin the oracle's outputs on seeded volumes, produced
by the engine's own deterministic generator (the SHA-256 of every volume is
stored and checked), so that GPU parity tests on any host compare against
the same numbers:

  small_cases.json  seconds:  tau / iterations / status of the oracle's
                    device-path and Eigen-path restatements (CG and BiCGSTAB,
                    FP64 at tol 1e-6 and 1e-10, FP32 at tol 1e-5) on small
                    volumes, plus an independent scipy.sparse assembly +
                    direct solve (spsolve) of the same operator.
  workloads.json    minutes:  FP64 tau at tol 1e-10 (the accuracy target) and
                    the reference-semantics FP64 iteration counts at tol 1e-6
                    for the benchmark volumes (64^3 spheres; 256^3 ellipsoids,
                    three directions).

  large (CPU, a minute): the 1024^3 large-volume spheres (seed 7, r = 10,
                    solid 0.65): the volume's SHA-256 and pore count, and the
                    oracle's connected-component labels of the pore phase
                    (label count, SHA-256 of the uint32 label array, SHA-256 of
                    the 7 x K face table).
  large_tau OUT     (GPU, about a minute): FP64 tau of that volume in x at tol
                    1e-10.  The oracle's stored-coefficient system of a 1024^3
                    volume needs 77 GB of host memory, so the GPU's FP64
                    Jacobi-PCG, the reference-semantics path that the parity
                    tests check against the oracle up to 256^3, stands in; the
                    record goes to OUT (JSON) and `merge OUT` adds it to
                    workloads.json.

Usage:  python tests/golden/make_golden.py [small|workloads|bicgstab1e-7|large|all]
        python tests/golden/make_golden.py large_tau OUT
        python tests/golden/make_golden.py merge OUT
"""
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fast_gb300 import build as _build  # noqa: E402

_build.build()
from fast_gb300 import volumes  # noqa: E402
from oracle import oracle as O  # noqa: E402


def sha(m):
    return hashlib.sha256(np.ascontiguousarray(m).tobytes()).hexdigest()


def scipy_tau(mask, d):
    """Independent restatement: scipy.sparse assembly of the same 7-point
    operator (arithmetic face mean, half-cell Dirichlet faces) + spsolve, and
    the tau plane-flux formula, all in FP64 with h = 1."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    nz, ny, nx = mask.shape
    N = mask.size
    D = np.where(mask.reshape(-1) > 0, np.float64(np.float32(0.001)), 1.0)
    k = d // 2
    sgn = 1 if d % 2 == 0 else -1
    res = (nx, ny, nz)
    idx = np.arange(N).reshape(nz, ny, nx)
    coords = [np.broadcast_to(np.arange(nx)[None, None, :], mask.shape).reshape(-1),
              np.broadcast_to(np.arange(ny)[None, :, None], mask.shape).reshape(-1),
              np.broadcast_to(np.arange(nz)[:, None, None], mask.shape).reshape(-1)]
    strides = (1, nx, nx * ny)
    rows, cols, vals = [], [], []
    diag = np.zeros(N)
    b = np.zeros(N)
    for ax in range(3):
        for s in (1, -1):
            c = coords[ax]
            inside = (c + s >= 0) & (c + s < res[ax])
            i = np.nonzero(inside)[0]
            j = i + s * strides[ax]
            f = (D[i] + D[j]) * 0.5
            rows.append(i); cols.append(j); vals.append(f)
            diag[i] -= f
            if ax == k:
                bnd = np.nonzero(~inside)[0]
                diag[bnd] -= 2.0 * D[bnd]
                conc = (1.0 if sgn > 0 else 0.0) if s == -1 else (0.0 if sgn > 0 else 1.0)
                b[bnd] -= 2.0 * D[bnd] * conc
    rows.append(np.arange(N)); cols.append(np.arange(N)); vals.append(diag)
    A = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))
    x = spl.spsolve(A.tocsc(), b)
    # tau
    c = coords[k]
    nxt = c + sgn
    valid = (nxt >= 0) & (nxt < res[k])
    cn = np.zeros(N)
    cn[valid] = x[np.nonzero(valid)[0] + sgn * strides[k]]
    dx = np.where(valid, 1.0, 0.5)
    coeff = np.where(mask.reshape(-1) == 0, np.float64(np.float32(1.0)), np.float64(np.float32(0.001)))
    flux = coeff * (x - cn) / dx
    phi = (mask == 0).sum() / N
    dimk = res[k]
    S = flux.sum()
    return float(phi / ((S / (N / dimk) / dimk) * dimk)) if phi > 0 else 0.0


def small_cases():
    cases = []
    specs = [
        ("spheres", (12, 14, 16), 1, 3.0, 0.5),
        ("spheres", (20, 18, 16), 2, 2.5, 0.6),
        ("spheres", (9, 17, 25), 3, 2.0, 0.4),
        ("ellipsoids", (16, 16, 16), 4, 5.0, 0.35),
        ("random", (7, 9, 11), 5, None, 0.5),
        ("random", (1, 6, 5), 6, None, 0.5),
        ("random", (4, 1, 3), 7, None, 0.3),
    ]
    for kind, shape, seed, r, frac in specs:
        if kind == "spheres":
            m = volumes.spheres(shape, seed, r, r, frac)
        elif kind == "ellipsoids":
            m = volumes.ellipsoids(shape, seed, r, 0.35, 0.55)
        else:
            m = ((np.random.default_rng(seed).random(shape) < frac) * 255).astype(np.uint8)
        entry = dict(kind=kind, shape=list(shape), seed=seed, r=r, frac=frac, sha256=sha(m),
                     pores=int((m == 0).sum()), results=[])
        for d in range(6):
            e = dict(dir=d, scipy_tau=scipy_tau(m, d))
            for sname, s in (("cg", O.CG), ("bicgstab", O.BICGSTAB)):
                for vname, v in (("device", O.DEVICE), ("eigen", O.EIGEN)):
                    for tol in (1e-6, 1e-10):
                        r_ = O.get_tortuosity(m, dir=d, solver=s, tol=tol, variant=v)
                        e[f"{sname}_{vname}_{tol:g}"] = [r_["tau"], r_["iters"], r_["status"]]
                r32 = O.get_tortuosity(m, dir=d, solver=s, tol=1e-5, dtype=np.float32)
                e[f"{sname}_f32_1e-05"] = [r32["tau"], r32["iters"], r32["status"]]
            entry["results"].append(e)
        if kind == "random":
            entry["volume"] = m.reshape(-1).tolist()
        cases.append(entry)
    with open(os.path.join(HERE, "small_cases.json"), "w") as f:
        json.dump(dict(generator="tests/golden/make_golden.py", cases=cases), f, indent=1)


def workloads():
    out = {}
    wl = [
        ("spheres64", dict(kind="spheres", shape=(64, 64, 64), seed=0, r=5.0, frac=0.60), [0]),
        ("ellipsoids256", dict(kind="ellipsoids", shape=(256, 256, 256), seed=1, a=12.0, aspect=0.35, frac=0.55),
         [0, 2, 4]),
    ]
    for name, spec, dirs in wl:
        if spec["kind"] == "spheres":
            m = volumes.spheres(spec["shape"], spec["seed"], spec["r"], spec["r"], spec["frac"])
        else:
            m = volumes.ellipsoids(spec["shape"], spec["seed"], spec["a"], spec["aspect"], spec["frac"])
        e = dict(spec=spec, sha256=sha(m), pores=int((m == 0).sum()), dirs={})
        for d in dirs:
            t0 = time.time()
            cg = O.get_tortuosity(m, dir=d, solver=O.CG, tol=1e-10, max_iter=100000)
            bi = O.get_tortuosity(m, dir=d, solver=O.BICGSTAB, tol=1e-10, max_iter=100000, variant=O.EIGEN)
            ref_cg = O.get_tortuosity(m, dir=d, solver=O.CG, tol=1e-6, max_iter=100000)
            ref_bi = O.get_tortuosity(m, dir=d, solver=O.BICGSTAB, tol=1e-6, max_iter=100000)
            e["dirs"][str(d)] = {
                "tau_cg_1e-10": cg["tau"], "iters_cg_1e-10": cg["iters"],
                "tau_bicgstab_eigen_1e-10": bi["tau"], "iters_bicgstab_eigen_1e-10": bi["iters"],
                "tau_cg_1e-6": ref_cg["tau"], "iters_cg_1e-6": ref_cg["iters"],
                "tau_bicgstab_1e-6": ref_bi["tau"], "iters_bicgstab_1e-6": ref_bi["iters"],
                "seconds": time.time() - t0}
            print(name, d, e["dirs"][str(d)], flush=True)
        out[name] = e
        with open(os.path.join(HERE, "workloads.json"), "w") as f:
            json.dump(dict(generator="tests/golden/make_golden.py", workloads=out), f, indent=1)


def workloads_bicgstab_1e7():
    """Adds FP64 BiCGSTAB (the GPU path's and Eigen's recurrences) at tol 1e-7 (the tolerance at
    which BiCGSTAB meets |dtau|/tau <= 1e-5 on the 256^3 workload) to
    workloads.json."""
    path = os.path.join(HERE, "workloads.json")
    with open(path) as f:
        doc = json.load(f)
    for name, e in doc["workloads"].items():
        spec = e["spec"]
        if spec["kind"] == "spheres":
            m = volumes.spheres(spec["shape"], spec["seed"], spec["r"], spec["r"], spec["frac"])
        else:
            m = volumes.ellipsoids(spec["shape"], spec["seed"], spec["a"], spec["aspect"], spec["frac"])
        assert sha(m) == e["sha256"]
        for d, rec in e["dirs"].items():
            r = O.get_tortuosity(m, dir=int(d), solver=O.BICGSTAB, tol=1e-7, max_iter=100000)
            rec["tau_bicgstab_1e-7"] = r["tau"]
            rec["iters_bicgstab_1e-7"] = r["iters"]
            re_ = O.get_tortuosity(m, dir=int(d), solver=O.BICGSTAB, tol=1e-7, max_iter=100000, variant=O.EIGEN)
            rec["tau_bicgstab_eigen_1e-7"] = re_["tau"]
            rec["iters_bicgstab_eigen_1e-7"] = re_["iters"]
            print(name, d, r["tau"], r["iters"], re_["tau"], re_["iters"], flush=True)
    with open(path, "w") as f:
        json.dump(doc, f, indent=1)


LARGE = dict(kind="spheres", shape=(1024, 1024, 1024), seed=7, r=10.0, frac=0.65)


def large_volume():
    return volumes.spheres(LARGE["shape"], LARGE["seed"], LARGE["r"], LARGE["r"], LARGE["frac"])


def large():
    """Volume hash, pore count and the oracle's labels of the 1024^3 volume."""
    path = os.path.join(HERE, "workloads.json")
    with open(path) as f:
        doc = json.load(f)
    m = large_volume()
    t0 = time.time()
    labels, n = O.ccl_label(m)
    table = O.ccl_boundary(labels, n)
    e = doc["workloads"].setdefault("spheres1024", {})
    e.update(spec=dict(LARGE, shape=list(LARGE["shape"])), sha256=sha(m), pores=int((m == 0).sum()),
             ccl={"num_labels": int(n), "labels_sha256": sha(labels), "boundary_sha256": sha(table),
                  "x_spanning": int((table[0] & table[1])[1:].sum()),
                  "seconds": time.time() - t0})
    e.setdefault("dirs", {})
    print("spheres1024", e["sha256"], e["pores"], e["ccl"], flush=True)
    with open(path, "w") as f:
        json.dump(doc, f, indent=1)


def large_tau(out):
    """FP64 tau of the 1024^3 volume in x at tol 1e-10 on the GPU (FP64
    Jacobi-PCG, reference semantics), written to `out`."""
    import torch
    import fast_gb300 as ft
    m = large_volume()
    h = sha(m)
    d = torch.from_numpy(m).cuda()
    del m
    p = ft.TortuosityParams(tolerance=1e-10, max_iter=200000, precision=ft.Precision.F64)
    t0 = time.time()
    r = ft.solve_directions_device(d.data_ptr(), LARGE["shape"], [ft.Dir.X_POS], p, ft.DSOLVER_CG)[0]
    torch.cuda.synchronize()
    rec = {"sha256": h, "dirs": {"0": {"tau_cg_1e-10": r.tau, "iters_cg_1e-10": int(r.iterations),
                                        "status_cg_1e-10": int(r.status), "solver_cg_1e-10": "GPU F64 Jacobi-PCG",
                                        "seconds": time.time() - t0}}}
    print(json.dumps(rec), flush=True)
    with open(out, "w") as f:
        json.dump(rec, f, indent=1)


def merge(frag):
    path = os.path.join(HERE, "workloads.json")
    with open(path) as f:
        doc = json.load(f)
    with open(frag) as f:
        rec = json.load(f)
    e = doc["workloads"]["spheres1024"]
    assert rec["sha256"] == e["sha256"], "the GPU host generated another volume"
    for d, v in rec["dirs"].items():
        e["dirs"].setdefault(d, {}).update(v)
    with open(path, "w") as f:
        json.dump(doc, f, indent=1)


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "all"
    if what == "large_tau":
        large_tau(sys.argv[2])
        sys.exit(0)
    if what == "merge":
        merge(sys.argv[2])
        sys.exit(0)
    if what == "large":
        large()
        sys.exit(0)
    if what in ("small", "all"):
        small_cases()
    if what in ("workloads", "all"):
        workloads()
    if what in ("bicgstab1e-7", "all"):
        workloads_bicgstab_1e7()
