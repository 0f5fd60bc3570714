"""CPU tests of the C ABI library: it builds and loads, exports every symbol
include/fasttau.h declares, its host-side logic (defaults, argument checks,
seeded generators) behaves, without launching any GPU work."""
import ctypes as C
import hashlib
import json
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def header_symbols():
    with open(os.path.join(ROOT, "include", "fasttau.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"FAST_API\s+[^;(]*?\b(fast_\w+)\s*\(", src)))


def test_header_symbols_exported(native):
    syms = header_symbols()
    assert "fast_tau_solve" in syms and "fast_porosity" in syms
    for s in syms:
        assert hasattr(native, s), f"{s} declared in include/fasttau.h but not exported"


def test_binding_covers_header():
    from fast_gb300 import _native
    for s in header_symbols():
        assert s in _native.SIGNATURES, f"{s} missing from the ctypes binding"


def test_params_init_defaults(native):
    from fast_gb300 import _native
    p = _native.fast_tau_params()
    native.fast_tau_params_init(C.byref(p))
    assert p.dir == 1                       # X_NEG (VolumeMeasures.h:21)
    assert p.solver == 0                    # BICGSTAB (VolumeMeasures.h:55)
    assert p.tolerance == 1e-6 and p.max_iter == 10000
    assert p.d0 == 1.0 and p.d1 == float(np.float32(0.001))
    assert p.porosity < 0


def test_argument_errors_without_gpu(native):
    """Argument checks run before any CUDA call and report the cause."""
    from fast_gb300 import _native
    p = _native.fast_tau_params()
    native.fast_tau_params_init(C.byref(p))
    tau = C.c_double(5.0)
    assert native.fast_tau_solve(None, 4, 4, 4, C.byref(p), C.byref(tau), None, None, None) == 2
    assert tau.value == 0.0
    m = np.zeros((4, 4, 4), np.uint8)
    mp = m.ctypes.data_as(C.c_void_p)
    assert native.fast_tau_solve(mp, -1, 4, 4, C.byref(p), None, None, None, None) == 8
    p.dir = 9
    assert native.fast_tau_solve(mp, 4, 4, 4, C.byref(p), None, None, None, None) == 8
    assert b"direction" in native.fast_last_error()
    native.fast_tau_params_init(C.byref(p))
    p.precision = 5
    assert native.fast_tau_solve(mp, 4, 4, 4, C.byref(p), None, None, None, None) == 8


def test_python_mirror_failure_returns_zero(native, capsys):
    import fast_gb300 as ft
    p = ft.TortuosityParams()
    assert ft.get_tortuosity(np.zeros((2, 2), np.uint8), p) == 0.0
    assert "uchar" in capsys.readouterr().err
    assert ft.get_tortuosity(np.zeros((2, 2, 2), np.float32), p) == 0.0


def test_generators_deterministic(native):
    from fast_gb300 import volumes
    a = volumes.spheres((20, 22, 24), seed=5, r_min=2.0, r_max=4.0, solid_fraction=0.5)
    b = volumes.spheres((20, 22, 24), seed=5, r_min=2.0, r_max=4.0, solid_fraction=0.5)
    assert np.array_equal(a, b)
    assert set(np.unique(a)) <= {0, 255}
    assert abs((a != 0).mean() - 0.5) < 0.01
    e = volumes.ellipsoids((16, 16, 16), seed=4, semi_major=5.0, aspect=0.35, solid_fraction=0.55)
    assert abs((e != 0).mean() - 0.55) < 0.01


def test_benchmark_volume_hash(native):
    """The 64^3 benchmark volume is bit-identical to the one the golden
    fixture was computed on (the generator uses no transcendental math)."""
    from fast_gb300 import volumes
    with open(os.path.join(HERE, "golden", "workloads.json")) as f:
        w = json.load(f)["workloads"]["spheres64"]
    s = w["spec"]
    m = volumes.spheres(tuple(s["shape"]), s["seed"], s["r"], s["r"], s["frac"])
    assert hashlib.sha256(m.tobytes()).hexdigest() == w["sha256"]


def test_ccl_argument_errors_without_gpu(native):
    """The labelling entry points check their arguments before any CUDA call."""
    n = C.c_uint32(0)
    assert native.fast_ccl_label(None, 4, 4, 4, 255, None, C.byref(n), None, 0) == 2
    m = np.zeros((4, 4, 4), np.uint8)
    mp = m.ctypes.data_as(C.c_void_p)
    assert native.fast_ccl_label(mp, 0, 4, 4, 255, None, C.byref(n), None, 0) == 8
    assert native.fast_ccl_label(mp, 4096, 4096, 256, 255, None, C.byref(n), None, 0) == 8
    assert b"4294967294" in native.fast_last_error()
    assert native.fast_ccl_label(mp, 4, 4, 4, 255, None, None, None, 0) == 8
    assert native.fast_ccl_label_device(None, 4, 4, 4, 255, None, C.byref(n), None, 0, None) == 8
    assert native.fast_ccl_boundary_device(None, 4, 4, 4, 3, None, None) == 8


def test_batch_argument_errors_without_gpu(native):
    from fast_gb300 import _native
    p = _native.fast_tau_params()
    native.fast_tau_params_init(C.byref(p))
    res = (_native.fast_tau_result * 2)()
    vols = (_native.fast_tau_volume * 2)()
    m = np.zeros((4, 4, 4), np.uint8)
    for v in vols:
        v.mask = m.ctypes.data
        v.nx = v.ny = v.nz = 4
        v.dir = 0
    assert native.fast_tau_solve_batch(None, 2, C.byref(p), res) == 8
    assert native.fast_tau_solve_batch(vols, 0, C.byref(p), res) == 8
    assert native.fast_tau_solve_batch(vols, 2000, C.byref(p), res) == 8
    vols[1].dir = 7
    assert native.fast_tau_solve_batch(vols, 2, C.byref(p), res) == 8
    assert b"volume 1" in native.fast_last_error()
    vols[1].dir = 0
    vols[1].mask = None
    assert native.fast_tau_solve_batch(vols, 2, C.byref(p), res) == 2


def test_ctx_argument_errors_without_gpu(native):
    from fast_gb300 import _native
    cfg = _native.fast_ctx_config()
    native.fast_ctx_config_init(C.byref(cfg))
    assert cfg.precision == 2 and cfg.chunk == 16 and cfg.max_inflight == 256 and cfg.tolerance == 1e-6
    h = C.c_void_p()
    assert native.fast_ctx_create(None, C.byref(h)) == 8
    cfg.chunk = 0
    assert native.fast_ctx_create(C.byref(cfg), C.byref(h)) == 8
    cfg.chunk = 16
    cfg.max_inflight = 5000
    assert native.fast_ctx_create(C.byref(cfg), C.byref(h)) == 8
    t = C.c_uint64(0)
    m = np.zeros((4, 4, 4), np.uint8)
    assert native.fast_ctx_submit(None, m.ctypes.data_as(C.c_void_p), 4, 4, 4, 0, 0, C.byref(t)) == 8
