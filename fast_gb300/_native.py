"""ctypes binding of libfasttau.so (the C ABI declared in include/fasttau.h).

The library is the only compute path: when it is missing or fails to load,
every entry point raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

_lock = threading.Lock()
_lib = None


class fast_tau_params(C.Structure):
    _fields_ = [
        ("dir", C.c_int32), ("solver", C.c_int32), ("precision", C.c_int32), ("face_mean", C.c_int32),
        ("tolerance", C.c_double), ("max_iter", C.c_uint64), ("d0", C.c_double), ("d1", C.c_double),
        ("porosity", C.c_double), ("verbose", C.c_int32), ("flags", C.c_int32),
    ]


class fast_tau_result(C.Structure):
    _fields_ = [
        ("tau", C.c_double), ("porosity", C.c_double), ("rel_residual", C.c_double),
        ("iterations", C.c_uint64), ("outer_steps", C.c_uint32), ("status", C.c_int32),
    ]


class fast_tau_volume(C.Structure):
    _fields_ = [("mask", C.c_void_p), ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
                ("dir", C.c_int32), ("reserved", C.c_int32)]


class fast_ctx_config(C.Structure):
    _fields_ = [("precision", C.c_int32), ("face_mean", C.c_int32), ("tolerance", C.c_double),
                ("max_iter", C.c_uint64), ("d0", C.c_double), ("d1", C.c_double), ("chunk", C.c_int32),
                ("max_inflight", C.c_int32), ("hbm_budget", C.c_uint64)]


class fast_ctx_completion(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("result", fast_tau_result), ("dir", C.c_int32), ("solver", C.c_int32),
                ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double)]


class fast_ctx_stats(C.Structure):
    _fields_ = [("pending", C.c_uint64), ("inflight", C.c_uint64), ("completed", C.c_uint64),
                ("admitted", C.c_uint64), ("steps", C.c_uint64), ("bytes_inflight", C.c_uint64),
                ("hbm_budget", C.c_uint64), ("now", C.c_double)]


K_COUNT = 16
KERNEL_NAMES = ["code", "init", "cg1", "cg2", "bi_restart", "bi1", "bi2", "bi3", "replace", "init64", "tau", "cgf"]
FLAG_PROFILE = 1
FLAG_REPLACE_FLOAT_FLOAT = 2


class fast_tau_stats(C.Structure):
    _fields_ = [
        ("launches", C.c_uint64), ("graph_replays", C.c_uint64), ("kernel_launches", C.c_uint64 * K_COUNT),
        ("kernel_ms", C.c_double * K_COUNT), ("profiled", C.c_int32), ("pad", C.c_int32),
    ]


# Every symbol include/fasttau.h declares, with its ctypes signature.
SIGNATURES = {
    "fast_tau_params_init": (None, [C.POINTER(fast_tau_params)]),
    "fast_tau_solve": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.POINTER(fast_tau_params),
                                 C.POINTER(C.c_double), C.POINTER(C.c_uint64), C.POINTER(C.c_double), C.c_void_p]),
    "fast_tau_solve_dirs": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.POINTER(fast_tau_params),
                                      C.c_int32, C.POINTER(C.c_int32), C.POINTER(fast_tau_result)]),
    "fast_tau_solve_dirs_device": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
                                             C.POINTER(fast_tau_params), C.c_int32, C.POINTER(C.c_int32),
                                             C.POINTER(fast_tau_result), C.c_void_p]),
    "fast_porosity": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.POINTER(C.c_double),
                                C.POINTER(C.c_uint64)]),
    "fast_tau_last_stats": (C.c_int, [C.POINTER(fast_tau_stats)]),
    "fast_tau_slab_depth": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_int32, C.c_int32,
                                      C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "fast_tau_set_slab_table": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.c_int32]),
    "fast_porosity_device_noalloc": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.POINTER(C.c_uint64),
                                               C.POINTER(C.c_double), C.c_void_p]),
    "fast_tau_solve_batch": (C.c_int, [C.POINTER(fast_tau_volume), C.c_int32, C.POINTER(fast_tau_params),
                                       C.POINTER(fast_tau_result)]),
    "fast_tau_solve_batch_device": (C.c_int, [C.POINTER(fast_tau_volume), C.c_int32, C.POINTER(fast_tau_params),
                                              C.POINTER(fast_tau_result), C.c_void_p]),
    "fast_ctx_config_init": (None, [C.POINTER(fast_ctx_config)]),
    "fast_ctx_create": (C.c_int, [C.POINTER(fast_ctx_config), C.POINTER(C.c_void_p)]),
    "fast_ctx_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_int32, C.c_int32,
                                  C.POINTER(C.c_uint64)]),
    "fast_ctx_poll": (C.c_int, [C.c_void_p, C.POINTER(fast_ctx_completion), C.c_int32, C.POINTER(C.c_int32)]),
    "fast_ctx_query": (C.c_int, [C.c_void_p, C.POINTER(fast_ctx_stats)]),
    "fast_ctx_destroy": (C.c_int, [C.c_void_p]),
    "fast_ccl_label": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_uint8, C.c_void_p,
                                 C.POINTER(C.c_uint32), C.c_void_p, C.c_uint64]),
    "fast_ccl_label_device": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_uint8, C.c_void_p,
                                        C.POINTER(C.c_uint32), C.c_void_p, C.c_uint64, C.c_void_p]),
    "fast_ccl_boundary_device": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_uint32, C.c_void_p,
                                           C.c_void_p]),
    "fast_tiff_folder_info": (C.c_int, [C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                        C.POINTER(C.c_int64)]),
    "fast_tiff_folder_read": (C.c_int, [C.c_char_p, C.c_void_p, C.c_uint64]),
    "fast_binarize": (C.c_int, [C.c_void_p, C.c_uint64, C.c_float]),
    "fast_binarize_device": (C.c_int, [C.c_void_p, C.c_uint64, C.c_float, C.c_void_p]),
    "fast_reactive_area": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_float,
                                     C.POINTER(C.c_double)]),
    "fast_reactive_area_device": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_float,
                                            C.POINTER(C.c_double), C.c_void_p]),
    "fast_reactive_area_tensor": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_float,
                                            C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "fast_reactive_area_tensor_device": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_float,
                                                   C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p]),
    "fast_reactive_area_mesh": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_float, C.c_void_p,
                                          C.c_uint64, C.POINTER(C.c_uint64)]),
    "fast_last_error": (C.c_char_p, []),
    "fast_version": (C.c_char_p, []),
    "fast_gen_spheres": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_uint64, C.c_double,
                                   C.c_double, C.c_double]),
    "fast_gen_ellipsoids": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_uint64, C.c_double,
                                      C.c_double, C.c_double]),
}


def lib_path() -> str:
    """The in-tree build, or FAST_TAU_LIB (another build of the same library,
    e.g. one compiled with FAST_TAU_BOUNDS_CHECK)."""
    return os.environ.get("FAST_TAU_LIB") or _build.LIB


def lib():
    """The loaded library.  Raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            path = lib_path()
            if not os.path.exists(path):
                raise RuntimeError(
                    f"libfasttau.so is not built ({path}); run `python -m fast_gb300.build` "
                    "or __graft_entry__.build() first")
            L = C.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def last_error() -> str:
    return lib().fast_last_error().decode(errors="replace")


def last_stats() -> dict:
    st = fast_tau_stats()
    lib().fast_tau_last_stats(C.byref(st))
    per = {}
    for k, name in enumerate(KERNEL_NAMES):
        n = int(st.kernel_launches[k])
        if n:
            per[name] = {"launches": n, "ms": float(st.kernel_ms[k])}
    return {"launches": int(st.launches), "graph_replays": int(st.graph_replays), "profiled": bool(st.profiled),
            "kernels": per}
