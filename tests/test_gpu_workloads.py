"""The seeded workload volumes against their golden records
(tests/golden/workloads.json), through the C ABI:

  * plain drop-in (64^3 spheres, seed 0, r 5, solid 0.60; x; FP64 Jacobi-PCG,
    tol 1e-6) through fast_tau_solve: tau within 1e-9 of the oracle's
    device-path CG at the same tolerance, the same iteration count, and within
    1e-5 of the oracle's FP64 tol-1e-10 tau;
  * the 256^3 ellipsoid volume (seed 1), x/y/z as three right-hand sides,
    MIXED BiCGSTAB at tol 1e-7: every direction within 1e-5 of the oracle's
    FP64 tol-1e-10 tau;
  * the 1024^3 spheres (seed 7, r 10, solid 0.65): connected-component labels
    of the pore phase bit-identical to the oracle's (label count, SHA-256 of
    the whole uint32 label array and of the 7 x K face table), and MIXED
    Jacobi-PCG in x at tol 1e-6 within 1e-5 of the FP64 tau at tol 1e-10.

Every volume is regenerated here and its SHA-256 checked against the record,
so all hosts compare the same bytes.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import fast_gb300 as ft
from fast_gb300 import volumes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu


def _golden(name):
    with open(os.path.join(ROOT, "tests", "golden", "workloads.json")) as f:
        return json.load(f)["workloads"][name]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _make(spec):
    if spec["kind"] == "spheres":
        return volumes.spheres(tuple(spec["shape"]), spec["seed"], spec["r"], spec["r"], spec["frac"])
    return volumes.ellipsoids(tuple(spec["shape"]), spec["seed"], spec["a"], spec["aspect"], spec["frac"])


def rel(a, b):
    return abs(a - b) / abs(b)


def test_plain_dropin_64_f64_cg_matches_oracle(gpu):
    g = _golden("spheres64")
    m = _make(g["spec"])
    assert _sha(m) == g["sha256"]
    rec = g["dirs"]["0"]
    p = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-6, max_iter=10000, precision=ft.Precision.F64)
    it = []
    tau = ft.get_tortuosity(m, p, ft.DSOLVER_CG, iterations_out=it)
    assert rel(tau, rec["tau_cg_1e-6"]) <= 1e-9
    assert it[0] == rec["iters_cg_1e-6"]
    assert rel(tau, rec["tau_cg_1e-10"]) <= 1e-5


def test_ellipsoids256_three_dirs_mixed_bicgstab_vs_fp64(gpu):
    g = _golden("ellipsoids256")
    m = _make(g["spec"])
    assert _sha(m) == g["sha256"]
    dirs = [ft.Dir.X_POS, ft.Dir.Y_POS, ft.Dir.Z_POS]
    p = ft.TortuosityParams(tolerance=1e-7, max_iter=10000, precision=ft.Precision.MIXED)
    res = ft.solve_directions(m, dirs, p, ft.DSOLVER_BICGSTAB)
    for r in res:
        assert r.status == ft.Status.OK
        assert rel(r.tau, g["dirs"][str(int(r.dir))]["tau_cg_1e-10"]) <= 1e-5, r


@pytest.fixture(scope="module")
def large():
    g = _golden("spheres1024")
    m = _make(g["spec"])
    assert _sha(m) == g["sha256"]
    assert int((m == 0).sum()) == g["pores"]
    return g, m


def test_large_volume_labels_bit_exact(gpu, large):
    from fast_gb300 import ccl
    g, m = large
    c = ccl.get_volume_ccl(m, background=255)
    assert c.num_labels == g["ccl"]["num_labels"]
    assert _sha(c.labels) == g["ccl"]["labels_sha256"]
    assert _sha(c.boundary_label_mask) == g["ccl"]["boundary_sha256"]
    assert int(c.get_dir_mask(ft.Dir.X_NEG, ft.Dir.X_POS)[1:].sum()) == g["ccl"]["x_spanning"]


def test_large_volume_mixed_cg_vs_fp64(gpu, large):
    g, m = large
    rec = g["dirs"]["0"]
    p = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-6, max_iter=100000, precision=ft.Precision.MIXED)
    r = ft.solve_directions(m, [ft.Dir.X_POS], p, ft.DSOLVER_CG)[0]
    assert r.status == ft.Status.OK
    assert rel(r.tau, rec["tau_cg_1e-10"]) <= 1e-5
