"""ctypes front end of the CPU oracle (tau_oracle.c, ccl_oracle.c, alpha_oracle.c).

TEST INFRASTRUCTURE ONLY.  tests/, the smoke check and bench.py's CPU
baseline leg use this module as the checker for the CUDA path; the product
package never imports it.

Every function restates a reference routine; the C sources cite the
reference file:line each one follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "liboracle.so")
_lock = threading.Lock()
_lib = None

# Status codes shared with the C ABI of the product library.
OK, BAD_ARG, NOMEM, NO_CONVERGENCE = 0, 1, 3, 4
DEVICE, EIGEN = 0, 1  # which reference solver variant to restate
BICGSTAB, CG = 0, 1   # fast::DiffusionSolverType order (VolumeMeasures.h:15-18)
X_POS, X_NEG, Y_POS, Y_NEG, Z_POS, Z_NEG = range(6)

# TauModule::getTau passes coeffs as a float vec2 {1.0, 0.001} (TauModule.h:70).
D0_F32 = float(np.float32(1.0))
D1_F32 = float(np.float32(0.001))


_GEN_SO = os.path.join(_HERE, "_build", "libvolgen.so")
_GEN_SRC = os.path.join(_HERE, os.pardir, "fast_gb300", "csrc", "gen.cpp")
_gen = None


def build(force: bool = False) -> str:
    """Compile the oracle and the volume generator with the Makefile (gcc,
    OpenMP; g++ for the generator)."""
    srcs = [os.path.join(_HERE, f) for f in ("tau_oracle.c", "tau_oracle_impl.h", "ccl_oracle.c", "alpha_oracle.c",
                                             "Makefile")] + [_GEN_SRC]
    if not force and os.path.exists(_SO) and os.path.exists(_GEN_SO):
        so_m = min(os.path.getmtime(_SO), os.path.getmtime(_GEN_SO))
        if all(os.path.getmtime(s) <= so_m for s in srcs):
            return _SO
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_SO)
            P = C.c_void_p
            i64, u64, f32, f64, i32 = C.c_int64, C.c_uint64, C.c_float, C.c_double, C.c_int
            for sfx in ("f64", "f32"):
                getattr(L, f"oracle_assemble_{sfx}").argtypes = [P, i64, i64, i64, i32, f64, f64, f32, P, P, P]
                getattr(L, f"oracle_assemble_{sfx}").restype = i32
                getattr(L, f"oracle_spmv_{sfx}").argtypes = [P, i64, i64, i64, P, P]
                getattr(L, f"oracle_residual_{sfx}").argtypes = [P, i64, i64, i64, P, P, P]
                getattr(L, f"oracle_solve_{sfx}").argtypes = [P, i64, i64, i64, P, P, i32, f64, u64, i32,
                                                                C.POINTER(u64), C.POINTER(f64)]
                getattr(L, f"oracle_solve_{sfx}").restype = i32
                getattr(L, f"oracle_tau_{sfx}").argtypes = [P, i64, i64, i64, i32, f32, f32, P, f64]
                getattr(L, f"oracle_tau_{sfx}").restype = f64
                getattr(L, f"oracle_get_tortuosity_{sfx}").argtypes = [
                    P, i64, i64, i64, i32, i32, f64, u64, f32, f32, f64, i32, P,
                    C.POINTER(u64), C.POINTER(f64), C.POINTER(i32)]
                getattr(L, f"oracle_get_tortuosity_{sfx}").restype = f64
            L.oracle_count_pores.argtypes = [P, i64]
            L.oracle_count_pores.restype = u64
            L.oracle_ccl_label.argtypes = [P, i64, i64, i64, C.c_uint8, P]
            L.oracle_ccl_label.restype = C.c_uint32
            L.oracle_ccl_boundary.argtypes = [P, i64, i64, i64, C.c_uint32, P]
            L.oracle_area_field.argtypes = [P, i64, i64, i64, f32]
            L.oracle_area_field.restype = f64
            L.oracle_mc_ntri.argtypes = [i32]
            L.oracle_mc_ntri.restype = i32
            _lib = L
    return _lib


def build_ref() -> None:
    """Compile the reference's own assembly rule into oracle/_ref/ where the
    reference's source tree is present (the Makefile's `ref-if-present`);
    elsewhere this does nothing."""
    subprocess.run(["make", "-s", "-C", _HERE, "ref-if-present"], check=True)


def _volgen():
    """libvolgen.so: the seeded generator without the CUDA library."""
    global _gen
    with _lock:
        if _gen is None:
            build()
            G = C.CDLL(_GEN_SO)
            G.fast_gen_spheres.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_uint64, C.c_double,
                                           C.c_double, C.c_double]
            G.fast_gen_ellipsoids.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.c_uint64, C.c_double,
                                              C.c_double, C.c_double]
            G.fast_gen_spheres.restype = G.fast_gen_ellipsoids.restype = C.c_int
            _gen = G
    return _gen


def gen_spheres(shape, seed, r_min, r_max, solid_fraction):
    """The same bytes as fast_gb300.volumes.spheres (same source file)."""
    nz, ny, nx = shape
    out = np.empty((nz, ny, nx), dtype=np.uint8)
    assert _volgen().fast_gen_spheres(_ptr(out), nx, ny, nz, seed, r_min, r_max, solid_fraction) == OK
    return out


def gen_ellipsoids(shape, seed, semi_major, aspect, solid_fraction):
    """The same bytes as fast_gb300.volumes.ellipsoids (same source file)."""
    nz, ny, nx = shape
    out = np.empty((nz, ny, nx), dtype=np.uint8)
    assert _volgen().fast_gen_ellipsoids(_ptr(out), nx, ny, nz, seed, semi_major, aspect, solid_fraction) == OK
    return out


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _dims(mask: np.ndarray):
    """Volumes are numpy arrays indexed [z, y, x] (x fastest, Types.h:30-32)."""
    assert mask.ndim == 3 and mask.dtype == np.uint8 and mask.flags.c_contiguous
    nz, ny, nx = mask.shape
    return nx, ny, nz


def _sfx(dtype):
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def assemble(mask, dir, dtype=np.float64, d0=D0_F32, d1=D1_F32):
    """Stored system (A[7, N], b, x0) as GenerateDiffusionLinearSystem* builds it."""
    nx, ny, nz = _dims(mask)
    N = nx * ny * nz
    A = np.empty((7, N), dtype=dtype)
    b = np.empty(N, dtype=dtype)
    x0 = np.empty(N, dtype=dtype)
    cell = np.float32(1.0) / np.float32(max(nx, ny, nz))
    st = getattr(lib(), f"oracle_assemble_{_sfx(dtype)}")(
        _ptr(mask), nx, ny, nz, dir, d0, d1, float(cell), _ptr(A), _ptr(b), _ptr(x0))
    assert st == OK
    return A, b, x0


def spmv(A, mask_shape, x):
    nz, ny, nx = mask_shape
    y = np.empty_like(x)
    getattr(lib(), f"oracle_spmv_{_sfx(x.dtype)}")(_ptr(A), nx, ny, nz, _ptr(x), _ptr(y))
    return y


def residual(A, mask_shape, x, b):
    nz, ny, nx = mask_shape
    r = np.empty_like(x)
    getattr(lib(), f"oracle_residual_{_sfx(x.dtype)}")(_ptr(A), nx, ny, nz, _ptr(x), _ptr(b), _ptr(r))
    return r


def solve(A, mask_shape, b, x0, solver=CG, tol=1e-6, max_iter=10000, variant=DEVICE):
    nz, ny, nx = mask_shape
    x = x0.copy()
    it = C.c_uint64(0)
    err = C.c_double(0)
    st = getattr(lib(), f"oracle_solve_{_sfx(x.dtype)}")(
        _ptr(A), nx, ny, nz, _ptr(b), _ptr(x), solver, tol, max_iter, variant, C.byref(it), C.byref(err))
    return x, int(st), int(it.value), float(err.value)


def tau_from_conc(mask, dir, conc, porosity, c0=D0_F32, c1=D1_F32):
    nx, ny, nz = _dims(mask)
    conc = np.ascontiguousarray(conc).reshape(-1)
    return float(getattr(lib(), f"oracle_tau_{_sfx(conc.dtype)}")(
        _ptr(mask), nx, ny, nz, dir, c0, c1, _ptr(conc), porosity))


def count_pores(mask) -> int:
    return int(lib().oracle_count_pores(_ptr(mask), mask.size))


def get_tortuosity(mask, dir=X_POS, solver=CG, tol=1e-6, max_iter=10000, dtype=np.float64,
                   porosity=-1.0, variant=DEVICE, return_conc=False, c0=D0_F32, c1=D1_F32):
    """getTortuosity<T> restated: returns dict(tau, status, iters, err[, conc])."""
    nx, ny, nz = _dims(mask)
    conc = np.empty(nx * ny * nz, dtype=dtype)
    it = C.c_uint64(0)
    err = C.c_double(0)
    st = C.c_int(0)
    tau = getattr(lib(), f"oracle_get_tortuosity_{_sfx(dtype)}")(
        _ptr(mask), nx, ny, nz, dir, solver, tol, max_iter, c0, c1, porosity, variant,
        _ptr(conc), C.byref(it), C.byref(err), C.byref(st))
    out = dict(tau=float(tau), status=int(st.value), iters=int(it.value), err=float(err.value))
    if return_conc:
        out["conc"] = conc.reshape(nz, ny, nx)
    return out


def ccl_label(vol, background=255):
    """(labels uint32 [z,y,x], num_labels) as VolumeCCL_Label returns them."""
    nx, ny, nz = _dims(vol)
    labels = np.empty(vol.shape, dtype=np.uint32)
    n = int(lib().oracle_ccl_label(_ptr(vol), nx, ny, nz, background, _ptr(labels)))
    assert n > 0
    return labels, n


def ccl_boundary(labels, num_labels):
    """uint8 [7, num_labels] face-membership table (VolumeCCL_BoundaryLabels)."""
    nz, ny, nx = labels.shape
    out = np.empty((7, num_labels), dtype=np.uint8)
    lib().oracle_ccl_boundary(_ptr(labels), nx, ny, nz, num_labels, _ptr(out))
    return out


def binarize(vol, threshold=1.0):
    """Volume::binarize on uint8 (fastlib/src/volume/Volume.cpp:478-486,
    kernelBinarizeUnsigned and launchBinarizeKernel in fastlib/src/cuda/
    Volume.cu:157-183): t = uchar(threshold*255); v < t -> 0, else 255
    (T(-1) for uchar).  The threshold is clamped to [0, 1] before the
    conversion."""
    t = float(np.float32(min(max(float(threshold), 0.0), 1.0)) * np.float32(255.0))
    t = int(t)
    v = np.asarray(vol, dtype=np.uint8)
    return np.where(v < t, 0, 255).astype(np.uint8)


def area_field(field, iso=0.5) -> float:
    """Marching-cubes area of the isovalue surface of a 0/1 field [z, y, x]
    (getVolumeArea + sum, VolumeSurface.cpp:10-36, VolumeMeasures.cpp:294-301)."""
    f = np.ascontiguousarray(field, dtype=np.uint8)
    nx, ny, nz = _dims(f)
    return float(lib().oracle_area_field(_ptr(f), nx, ny, nz, float(iso)))


def reactive_area(mask, iso=0.5) -> float:
    """getReactiveAreaDensity(mask, mask.dim(), iso) on a 0/255 mask."""
    return area_field(np.asarray(mask) != 0, iso)


def reactive_area_tensor(mask, iso=0.5):
    """getVolumeCCL(mask, 255) + getReactiveAreaDensityTensor: for each Dir d
    the area of the pore components (voxels != 255) touching face d
    (generateBoundaryConnectedVolume, VolumeSegmentation.cpp:66-90)."""
    mask = np.ascontiguousarray(mask, dtype=np.uint8)
    labels, n = ccl_label(mask, 255)
    table = ccl_boundary(labels, n)
    return [area_field(table[d][labels], iso) for d in range(6)]

