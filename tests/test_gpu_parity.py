"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Tolerances:
  * F64 CG, same algorithm and tolerance as the oracle: |dtau|/tau <= 1e-9 at
    tol 1e-10 and <= 1e-7 at tol 1e-6 (the two runs differ only in rounding);
    iteration counts within +-2.
  * F64 BiCGSTAB: its non-symmetric recurrences amplify rounding, so the two
    runs stop at different iterates of equal residual: |dtau|/tau <= 1e-8 at
    tol 1e-10 and <= 1e-5 at tol 1e-6; iteration counts within 50 %.
  * F32 vs the float oracle at tol 1e-5: |dtau|/tau <= 1e-4.
  * MIXED (FP32 iterations + FP64 residual replacement) at tol 1e-7 vs the
    FP64 oracle at tol 1e-10: |dtau|/tau <= 1e-5 (the engine's accuracy
    contract); at tol 1e-10, far below what FP32 alone can reach, within 1e-8
    (the FP64 residual replacement carries the solve there).  A
    relative residual of 1e-6 is not enough for 1e-5 in tau on contrast-1000
    media: the reference's own FP64 BiCGSTAB at tol 1e-6 misses it by 3x on
    the 256^3 benchmark volume.
"""
import ctypes as C
import os

import numpy as np
import pytest

import fast_gb300 as ft
from fast_gb300 import volumes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu

OSOLVER = {ft.DSOLVER_CG: 1, ft.DSOLVER_BICGSTAB: 0}


def rel(a, b):
    return abs(a - b) / abs(b)


def _vol(shape, seed, frac=0.5, r=3.0):
    return volumes.spheres(shape, seed=seed, r_min=r, solid_fraction=frac)


@pytest.mark.parametrize("solver", [ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB])
@pytest.mark.parametrize("d", list(range(6)))
def test_f64_matches_oracle_all_dirs(gpu, oracle, solver, d):
    mask = _vol((18, 21, 24), seed=11 + d)
    p = ft.TortuosityParams(dir=ft.Dir(d), tolerance=1e-10)
    it = []
    tau = ft.get_tortuosity(mask, p, solver, iterations_out=it)
    ref = oracle.get_tortuosity(mask, dir=d, solver=OSOLVER[solver], tol=1e-10)
    assert ref["status"] == 0
    if solver == ft.DSOLVER_CG:
        assert rel(tau, ref["tau"]) <= 1e-9
        assert abs(it[0] - ref["iters"]) <= 2
    else:
        assert rel(tau, ref["tau"]) <= 1e-8
        assert abs(it[0] - ref["iters"]) <= 0.5 * ref["iters"] + 5


@pytest.mark.parametrize("solver", [ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB])
def test_f64_reference_tolerance(gpu, oracle, solver):
    """The reference's CLI setting: tol 1e-6, 10000 iterations."""
    mask = _vol((40, 40, 40), seed=5, frac=0.6, r=4.0)
    p = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-6)
    it = []
    tau = ft.get_tortuosity(mask, p, solver, iterations_out=it)
    ref = oracle.get_tortuosity(mask, dir=0, solver=OSOLVER[solver], tol=1e-6)
    if solver == ft.DSOLVER_CG:
        assert rel(tau, ref["tau"]) <= 1e-7
        assert abs(it[0] - ref["iters"]) <= 2
    else:
        assert rel(tau, ref["tau"]) <= 1e-5
        assert abs(it[0] - ref["iters"]) <= 0.5 * ref["iters"] + 5


@pytest.mark.parametrize("solver", [ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB])
def test_f32_matches_float_oracle(gpu, oracle, solver):
    mask = _vol((24, 20, 28), seed=7)
    p = ft.TortuosityParams(dir=ft.Dir.Y_POS, tolerance=1e-5, precision=ft.Precision.F32)
    tau = ft.get_tortuosity(mask, p, solver)
    ref = oracle.get_tortuosity(mask, dir=2, solver=OSOLVER[solver], tol=1e-5, dtype=np.float32)
    assert ref["status"] == 0
    assert rel(tau, ref["tau"]) <= 1e-4


@pytest.mark.parametrize("ff", [False, True], ids=["x64_fp64", "x64_float_float"])
@pytest.mark.parametrize("solver", [ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB])
def test_mixed_within_1e5_of_fp64_oracle(gpu, oracle, solver, ff):
    mask = _vol((48, 40, 36), seed=9, frac=0.6, r=4.0)
    for d in (0, 3, 4):
        p = ft.TortuosityParams(dir=ft.Dir(d), tolerance=1e-7, precision=ft.Precision.MIXED,
                                replace_float_float=ff)
        tau = ft.get_tortuosity(mask, p, solver)
        ref = oracle.get_tortuosity(mask, dir=d, solver=1, tol=1e-10)
        assert rel(tau, ref["tau"]) <= 1e-5, (d, tau, ref["tau"])


@pytest.mark.parametrize("ff", [False, True], ids=["x64_fp64", "x64_float_float"])
@pytest.mark.parametrize("solver", [ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB])
def test_mixed_reaches_fp64_accuracy(gpu, oracle, solver, ff):
    mask = _vol((40, 36, 44), seed=21, frac=0.55, r=3.5)
    for d in (1, 2, 5):
        p = ft.TortuosityParams(dir=ft.Dir(d), tolerance=1e-10, precision=ft.Precision.MIXED,
                                replace_float_float=ff)
        res = ft.solve_directions(mask, [ft.Dir(d)], p, solver)[0]
        assert res.status == ft.Status.OK, res
        assert res.rel_residual <= 1e-10
        assert res.outer_steps >= 2  # the FP64 replacement ran beyond the first setup
        ref = oracle.get_tortuosity(mask, dir=d, solver=1, tol=1e-10)
        assert rel(res.tau, ref["tau"]) <= 1e-8, (d, res.tau, ref["tau"])


def test_mixed_multi_direction_equals_single(gpu):
    mask = _vol((30, 26, 34), seed=23, frac=0.5, r=3.0)
    dirs = [ft.Dir.X_POS, ft.Dir.Y_NEG, ft.Dir.Z_POS]
    for solver in (ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB):
        p = ft.TortuosityParams(tolerance=1e-8, precision=ft.Precision.MIXED)
        multi = ft.solve_directions(mask, dirs, p, solver)
        for d, r in zip(dirs, multi):
            single = ft.solve_directions(mask, [d], p, solver)[0]
            # the right-hand sides of one launch never interact: bit-identical
            assert (r.tau, r.iterations, r.outer_steps) == (single.tau, single.iterations, single.outer_steps)


def test_known_answers(gpu):
    # all pore: tau = 1 in every direction
    m = np.zeros((6, 7, 9), np.uint8)
    for d in range(6):
        p = ft.TortuosityParams(dir=ft.Dir(d), tolerance=1e-12)
        assert abs(ft.get_tortuosity(m, p, ft.DSOLVER_CG) - 1.0) < 1e-9
    # all solid: porosity 0 -> tau 0
    m = np.full((5, 5, 5), 255, np.uint8)
    p = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-10)
    assert ft.get_tortuosity(m, p, ft.DSOLVER_CG) == 0.0
    # parallel layers: tau = phi / (phi + (1 - phi) D1)
    m = np.zeros((6, 8, 12), np.uint8)
    m[:, 2:5, :] = 255
    phi = (m == 0).mean()
    d1 = float(np.float32(0.001))
    p = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-12)
    assert rel(ft.get_tortuosity(m, p, ft.DSOLVER_CG), phi / (phi + (1 - phi) * d1)) < 1e-9


@pytest.mark.parametrize("zc", [3, 64, 1000])
def test_slab_depths_match_oracle(gpu, oracle, monkeypatch, zc):
    """Any slab depth (an odd one, the tuner's largest candidate, one above
    the volume's planes) gives the oracle's tau in every precision: the
    depth changes only the summation order of the partial sums."""
    monkeypatch.setenv("FAST_TAU_ZC", str(zc))
    mask = _vol((70, 19, 33), seed=29)
    for d in (0, 4, 5):
        ref = oracle.get_tortuosity(mask, dir=d, solver=1, tol=1e-10)
        assert ref["status"] == 0
        for solver in (ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB):
            for prec, bound in ((ft.Precision.F64, 1e-8), (ft.Precision.MIXED, 1e-5)):
                tol = 1e-10 if prec == ft.Precision.F64 else 1e-7
                p = ft.TortuosityParams(dir=ft.Dir(d), tolerance=tol, precision=prec)
                tau = ft.get_tortuosity(mask, p, solver)
                assert rel(tau, ref["tau"]) <= bound, (zc, d, solver, prec, tau, ref["tau"])


def test_tuned_depths_match_oracle(gpu, oracle, monkeypatch):
    """Volumes whose size classes select different tuned depths (2 to 64
    planes) match the oracle with the built-in table."""
    monkeypatch.delenv("FAST_TAU_ZC", raising=False)
    from fast_gb300 import autotune as at
    seen = set()
    for shape in ((40, 40, 40), (128, 64, 64), (256, 64, 64)):
        mask = _vol(shape, seed=sum(shape))
        ref = oracle.get_tortuosity(mask, dir=0, solver=1, tol=1e-10)
        for solver in (ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB):
            seen.add(at.slab_depth(shape, 1, ft.Precision.MIXED, solver)[0])
            p = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-7, precision=ft.Precision.MIXED)
            tau = ft.get_tortuosity(mask, p, solver)
            assert rel(tau, ref["tau"]) <= 1e-5, (shape, solver, tau, ref["tau"])
    assert len(seen) >= 2


@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 5, 1), (3, 1, 1), (1, 1, 7), (2, 3, 1), (33, 9, 65)])
def test_edge_shapes(gpu, oracle, shape):
    rng = np.random.default_rng(sum(shape))
    mask = ((rng.random(shape) < 0.4) * 255).astype(np.uint8)
    for d in range(6):
        for solver in (ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB):
            p = ft.TortuosityParams(dir=ft.Dir(d), tolerance=1e-11)
            tau = ft.get_tortuosity(mask, p, solver)
            ref = oracle.get_tortuosity(mask, dir=d, solver=OSOLVER[solver], tol=1e-11)
            if ref["status"] != 0:
                continue
            if ref["tau"] == 0.0:
                assert tau == 0.0
            else:
                assert rel(tau, ref["tau"]) <= 1e-7, (shape, d, solver, tau, ref)


@pytest.mark.parametrize("shape", [(1, 5, 1), (3, 1, 1), (2, 3, 1), (5, 3, 70), (7, 17, 9), (33, 9, 65),
                                   (4, 12, 130)])
def test_mixed_edge_shapes(gpu, oracle, shape):
    """MIXED (the FP32 sweeps with two rows per thread, the full-tile and the
    edge-tile plane loops, the FP64 replacement) on one-voxel axes, rows and
    columns that fill no tile, and tiles whose second thread row lies past
    the volume, in every direction: within 1e-6 of the oracle's FP64 CG at
    tol 1e-11, solved to tol 1e-10."""
    rng = np.random.default_rng(7 + sum(shape))
    mask = ((rng.random(shape) < 0.35) * 255).astype(np.uint8)
    for d in range(6):
        ref = oracle.get_tortuosity(mask, dir=d, solver=1, tol=1e-11)
        if ref["status"] != 0:
            continue
        for solver in (ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB):
            p = ft.TortuosityParams(dir=ft.Dir(d), tolerance=1e-10, precision=ft.Precision.MIXED)
            tau = ft.get_tortuosity(mask, p, solver)
            if ref["tau"] == 0.0:
                assert tau == 0.0, (shape, d, solver, tau)
            else:
                assert rel(tau, ref["tau"]) <= 1e-6, (shape, d, solver, tau, ref)


def test_concentration_output(gpu, oracle):
    mask = _vol((16, 18, 20), seed=4)
    p = ft.TortuosityParams(dir=ft.Dir.Z_NEG, tolerance=1e-11)
    conc = np.zeros(mask.shape, np.float64)
    ft.get_tortuosity(mask, p, ft.DSOLVER_CG, concentration_output=conc)
    ref = oracle.get_tortuosity(mask, dir=5, solver=1, tol=1e-11, return_conc=True)
    assert np.max(np.abs(conc - ref["conc"])) < 1e-8


@pytest.mark.parametrize("ff", [False, True], ids=["x64_fp64", "x64_float_float"])
def test_mixed_concentration_output(gpu, oracle, ff):
    """The MIXED iterate handed out as FP64 (read directly, or widened from
    float-float pairs) equals the oracle's field at a tight tolerance."""
    mask = _vol((16, 18, 20), seed=4)
    p = ft.TortuosityParams(dir=ft.Dir.Y_NEG, tolerance=1e-10, precision=ft.Precision.MIXED,
                            replace_float_float=ff)
    conc = np.zeros(mask.shape, np.float64)
    tau = ft.get_tortuosity(mask, p, ft.DSOLVER_BICGSTAB, concentration_output=conc)
    ref = oracle.get_tortuosity(mask, dir=3, solver=1, tol=1e-11, return_conc=True)
    assert rel(tau, ref["tau"]) <= 1e-8
    assert np.max(np.abs(conc - ref["conc"])) < 1e-7


def test_multi_direction_matches_single(gpu):
    mask = _vol((30, 26, 22), seed=21)
    p = ft.TortuosityParams(tolerance=1e-9)
    dirs = [ft.Dir.X_POS, ft.Dir.Y_POS, ft.Dir.Z_POS]
    res = ft.solve_directions(mask, dirs, p, ft.DSOLVER_BICGSTAB)
    for r, d in zip(res, dirs):
        p1 = ft.TortuosityParams(dir=d, tolerance=1e-9)
        it = []
        t1 = ft.get_tortuosity(mask, p1, ft.DSOLVER_BICGSTAB, iterations_out=it)
        assert r.status == ft.Status.OK
        assert r.tau == t1 and r.iterations == it[0]   # identical arithmetic, deterministic reductions


def test_porosity(gpu):
    mask = _vol((17, 19, 23), seed=2)
    assert ft.tau.get_pore_count(mask) == int((mask == 0).sum())


def test_non_convergence_and_errors(gpu):
    mask = _vol((20, 20, 20), seed=1)
    p = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-10, max_iter=1)
    it = []
    assert ft.get_tortuosity(mask, p, ft.DSOLVER_CG, iterations_out=it) == 0.0
    assert it[0] == 1
    from fast_gb300 import _native
    L = _native.lib()
    prm = _native.fast_tau_params()
    L.fast_tau_params_init(C.byref(prm))
    tau = C.c_double(1.0)
    # NULL mask -> NO_HOST_DATA; zero dims -> BAD_ARG; bad solver -> BAD_ARG
    assert L.fast_tau_solve(None, 4, 4, 4, C.byref(prm), C.byref(tau), None, None, None) == ft.Status.NO_HOST_DATA
    assert tau.value == 0.0
    m = np.zeros((4, 4, 4), np.uint8)
    assert L.fast_tau_solve(m.ctypes.data_as(C.c_void_p), 0, 4, 4, C.byref(prm), None, None, None, None) == ft.Status.BAD_ARG
    prm.solver = 7
    assert L.fast_tau_solve(m.ctypes.data_as(C.c_void_p), 4, 4, 4, C.byref(prm), None, None, None, None) == ft.Status.BAD_ARG
    assert b"solver" in L.fast_last_error()


@pytest.mark.gpu
def test_mixed_cg_one_sweep_option(gpu, oracle, tmp_path):
    """The opt-in one-sweep MIXED CG (FAST_TAU_CG_FUSED=1, read once per
    process, hence a child process) converges to the FP64 oracle's tau."""
    import subprocess
    import sys
    m = np.empty((40, 44, 48), np.uint8)
    assert gpu.fast_gen_spheres(m.ctypes.data_as(C.c_void_p), 48, 44, 40, 21, 3.0, 5.0, 0.5) == 0
    np.save(tmp_path / "m.npy", m)
    code = (
        "import sys, numpy as np; sys.path.insert(0, %r)\n"
        "import fast_gb300 as ft\n"
        "m = np.load(%r)\n"
        "p = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-8, precision=ft.Precision.MIXED)\n"
        "print(ft.get_tortuosity(m, p, ft.DSOLVER_CG))\n" % (ROOT, str(tmp_path / "m.npy")))
    env = dict(os.environ, FAST_TAU_CG_FUSED="1")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr
    tau = float(r.stdout.strip().splitlines()[-1])
    ref = oracle.get_tortuosity(m, dir=0, tol=1e-10)
    assert ref["status"] == 0
    assert rel(tau, ref["tau"]) <= 1e-5
