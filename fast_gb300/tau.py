"""Host-side mirror of fastlib's tortuosity API, served by libfasttau.so.

Same names, argument meaning and failure behaviour as
fastlib/include/fastlib/volume/VolumeMeasures.h:15-61:

* ``get_tortuosity(mask, params, solver_type, concentration_output,
  iterations_out)`` returns tau, or 0.0 with a message on stderr on any
  failure (VolumeMeasures.cpp:50-58, 100, 104-125, 157-159);
* ``get_porosity(mask)`` is the fraction of zero voxels;
* ``Dir``, ``DiffusionSolverType`` and ``TortuosityParams`` carry the
  reference's enum values and defaults.

Volumes are numpy uint8 arrays indexed ``[z, y, x]`` (x fastest in memory,
fastlib/include/fastlib/utility/Types.h:30-32), or ``Volume`` objects.
"""
from __future__ import annotations

import ctypes as C
import sys
from dataclasses import dataclass, field
from enum import IntEnum
from typing import List, Optional, Sequence

import numpy as np

from . import _native


class Dir(IntEnum):
    """enum Dir (fastlib/include/fastlib/utility/PrimitiveTypes.h:142-150)."""
    X_POS = 0
    X_NEG = 1
    Y_POS = 2
    Y_NEG = 3
    Z_POS = 4
    Z_NEG = 5
    DIR_NONE = 6


def get_dir_index(d: Dir) -> int:
    return int(d) // 2


def get_dir_sgn(d: Dir) -> int:
    return -((int(d) % 2) * 2 - 1)


class DiffusionSolverType(IntEnum):
    """enum DiffusionSolverType (VolumeMeasures.h:15-18)."""
    DSOLVER_BICGSTAB = 0
    DSOLVER_CG = 1


DSOLVER_BICGSTAB = DiffusionSolverType.DSOLVER_BICGSTAB
DSOLVER_CG = DiffusionSolverType.DSOLVER_CG


class Precision(IntEnum):
    """F64/F32: the reference's `-p double` / `-p float`; MIXED: FP32 Krylov
    iterations on a correction of an FP64 iterate, with FP64 true-residual
    replacement and an FP64 convergence test."""
    F64 = 0
    F32 = 1
    MIXED = 2


class FaceMean(IntEnum):
    ARITHMETIC = 0   # the reference (Diffusion.cu:47-53)
    HARMONIC = 1     # opt-in, never used for parity


class Status(IntEnum):
    OK = 0
    BAD_TYPE = 1
    NO_HOST_DATA = 2
    NOMEM = 3
    NO_CONVERGENCE = 4
    DIVERGED = 5
    CUDA_ERROR = 6
    TIMEOUT = 7
    BAD_ARG = 8
    IO_ERROR = 9


def _f32(v: float) -> float:
    return float(np.float32(v))


@dataclass
class TortuosityParams:
    """TortuosityParams (VolumeMeasures.h:20-34).  ``coeffs`` is a float vec2
    in the reference, so its values are rounded to float32."""
    dir: Dir = Dir.X_NEG
    coeffs: tuple = (_f32(1.0), _f32(0.001))
    tolerance: float = 1e-6
    max_iter: int = 10000
    verbose: bool = False
    oversubscribe_gpu_memory: bool = False
    use_non_uniform: bool = False
    porosity_precomputed: bool = False
    porosity: float = -1.0
    on_device: bool = True     # accepted for compatibility; the engine always solves on the GPU
    cpu_threads: int = -1
    # engine extensions
    precision: Precision = Precision.F64
    face_mean: FaceMean = FaceMean.ARITHMETIC
    profile: bool = False      # time every kernel launch (see _native.last_stats)
    # MIXED: float-float iterate and replacement residual instead of FP64 (opt-in)
    replace_float_float: bool = False

    def to_c(self, solver: DiffusionSolverType) -> _native.fast_tau_params:
        p = _native.fast_tau_params()
        p.dir = int(self.dir)
        p.solver = int(solver)
        p.precision = int(self.precision)
        p.face_mean = int(self.face_mean)
        p.tolerance = float(self.tolerance)
        p.max_iter = int(self.max_iter)
        p.d0 = _f32(self.coeffs[0])
        p.d1 = _f32(self.coeffs[1])
        p.porosity = float(self.porosity) if self.porosity_precomputed else -1.0
        p.verbose = 1 if self.verbose else 0
        p.flags = (_native.FLAG_PROFILE if self.profile else 0) | \
            (_native.FLAG_REPLACE_FLOAT_FLOAT if self.replace_float_float else 0)
        return p


class Volume:
    """Minimal fast::Volume stand-in: a host uint8 voxel array with dims
    (Volume.h:18-105; only what the tortuosity path reads)."""

    TYPE_UCHAR = 2  # PrimitiveType (PrimitiveTypes.h:11-24)

    def __init__(self, data: np.ndarray, type: int = TYPE_UCHAR):
        self.data = data
        self._type = type

    def dim(self):
        nz, ny, nx = self.data.shape
        return (nx, ny, nz)

    def type(self) -> int:
        return self._type if self.data.dtype == np.uint8 else -1

    def total_elems(self) -> int:
        return int(self.data.size)

    def sum_zero_elems(self) -> int:
        return get_pore_count(self.data)

    def binarize(self, threshold: float = 1.0) -> None:
        """Volume::binarize (Volume.cpp:478-486): v < uchar(threshold*255)
        -> 0, else 255, on the GPU (fast_binarize), in place."""
        if self.type() != Volume.TYPE_UCHAR:
            raise TypeError("binarize reads uint8 volumes")
        arr = np.ascontiguousarray(self.data)
        st = _native.lib().fast_binarize(arr.ctypes.data_as(C.c_void_p), arr.size, float(threshold))
        if st != Status.OK:
            raise RuntimeError(f"binarize failed ({Status(st).name}): {_native.last_error()}")
        self.data = arr


@dataclass
class TauResult:
    tau: float
    porosity: float
    rel_residual: float
    iterations: int
    outer_steps: int
    status: Status
    dir: Dir = Dir.X_POS
    message: str = ""


def _as_mask(mask):
    if isinstance(mask, Volume):
        if mask.type() != Volume.TYPE_UCHAR:
            return None
        mask = mask.data
    if not isinstance(mask, np.ndarray) or mask.dtype != np.uint8 or mask.ndim != 3:
        return None
    return np.ascontiguousarray(mask)


def _dims(m: np.ndarray):
    nz, ny, nx = m.shape
    return nx, ny, nz


def get_pore_count(mask) -> int:
    m = _as_mask(mask)
    if m is None:
        raise TypeError("mask must be a 3-D uint8 array [z, y, x]")
    nx, ny, nz = _dims(m)
    L = _native.lib()
    phi = C.c_double(0)
    cnt = C.c_uint64(0)
    st = L.fast_porosity(m.ctypes.data_as(C.c_void_p), nx, ny, nz, C.byref(phi), C.byref(cnt))
    if st != 0:
        raise RuntimeError(f"fast_porosity: {_native.last_error()}")
    return int(cnt.value)


def get_porosity(mask, dtype=np.float64) -> float:
    """getPorosity<T> (VolumeMeasures.cpp:289-292): T(#zero voxels)/T(N)."""
    m = _as_mask(mask)
    if m is None:
        raise TypeError("mask must be a 3-D uint8 array [z, y, x]")
    cnt = get_pore_count(m)
    return float(dtype(cnt) / dtype(m.size))


def get_tortuosity(mask, params: TortuosityParams, solver_type: DiffusionSolverType = DSOLVER_BICGSTAB,
                   concentration_output: Optional[np.ndarray] = None,
                   iterations_out: Optional[list] = None) -> float:
    """getTortuosity<T> (VolumeMeasures.cpp:42-285).  Returns tau, or 0.0 on
    failure with the cause on stderr.  ``concentration_output`` (optional) is
    a float64 (F64/MIXED) or float32 (F32) array of the mask's shape that
    receives the concentration field; ``iterations_out`` (optional list)
    receives the iteration count in element 0."""
    m = _as_mask(mask)
    if m is None:
        print("Mask must by type uchar", file=sys.stderr)
        return 0.0
    if params.use_non_uniform:
        print("useNonUniform is not supported by the GPU engine", file=sys.stderr)
        return 0.0
    nx, ny, nz = _dims(m)
    p = params.to_c(solver_type)
    tau = C.c_double(0)
    it = C.c_uint64(0)
    err = C.c_double(0)
    conc_ptr = None
    if concentration_output is not None:
        want = np.float32 if params.precision == Precision.F32 else np.float64
        if (concentration_output.dtype != want or concentration_output.shape != m.shape
                or not concentration_output.flags.c_contiguous):
            print("concentration output must be a contiguous %s array of the mask's shape" % np.dtype(want).name,
                  file=sys.stderr)
            return 0.0
        conc_ptr = concentration_output.ctypes.data_as(C.c_void_p)
    st = _native.lib().fast_tau_solve(m.ctypes.data_as(C.c_void_p), nx, ny, nz, C.byref(p), C.byref(tau),
                                      C.byref(it), C.byref(err), conc_ptr)
    if iterations_out is not None:
        if len(iterations_out):
            iterations_out[0] = int(it.value)
        else:
            iterations_out.append(int(it.value))
    if st != 0:
        print(_native.last_error(), file=sys.stderr)
        return 0.0
    return float(tau.value)


def solve_directions(mask, dirs: Sequence[Dir], params: TortuosityParams,
                     solver_type: DiffusionSolverType = DSOLVER_BICGSTAB) -> List[TauResult]:
    """Several directions of one volume as multiple right-hand sides sharing
    the device-resident phase field (one launch per solver step for all)."""
    m = _as_mask(mask)
    if m is None:
        raise TypeError("mask must be a 3-D uint8 array [z, y, x]")
    nx, ny, nz = _dims(m)
    p = params.to_c(solver_type)
    n = len(dirs)
    arr = (C.c_int32 * n)(*[int(d) for d in dirs])
    res = (_native.fast_tau_result * n)()
    st = _native.lib().fast_tau_solve_dirs(m.ctypes.data_as(C.c_void_p), nx, ny, nz, C.byref(p), n, arr, res)
    msg = _native.last_error() if st != 0 else ""
    if st not in (0, Status.NO_CONVERGENCE, Status.DIVERGED):
        raise RuntimeError(f"fast_tau_solve_dirs: {msg}")
    return [TauResult(r.tau, r.porosity, r.rel_residual, int(r.iterations), int(r.outer_steps), Status(r.status),
                      Dir(d), msg) for r, d in zip(res, dirs)]


def solve_directions_device(dev_ptr: int, shape, dirs: Sequence[Dir], params: TortuosityParams,
                            solver_type: DiffusionSolverType = DSOLVER_BICGSTAB, stream: int = 0) -> List[TauResult]:
    """As solve_directions on a device-resident uint8 mask (a device pointer,
    e.g. ``torch_tensor.data_ptr()``) of ``shape = (nz, ny, nx)``."""
    nz, ny, nx = shape
    p = params.to_c(solver_type)
    n = len(dirs)
    arr = (C.c_int32 * n)(*[int(d) for d in dirs])
    res = (_native.fast_tau_result * n)()
    st = _native.lib().fast_tau_solve_dirs_device(C.c_void_p(dev_ptr), nx, ny, nz, C.byref(p), n, arr, res,
                                                  C.c_void_p(stream) if stream else None)
    msg = _native.last_error() if st != 0 else ""
    if st not in (0, Status.NO_CONVERGENCE, Status.DIVERGED):
        raise RuntimeError(f"fast_tau_solve_dirs_device: {msg}")
    return [TauResult(r.tau, r.porosity, r.rel_residual, int(r.iterations), int(r.outer_steps), Status(r.status),
                      Dir(d), msg) for r, d in zip(res, dirs)]


def _batch_results(res, vols_dirs, msg):
    return [TauResult(r.tau, r.porosity, r.rel_residual, int(r.iterations), int(r.outer_steps), Status(r.status),
                      Dir(d), msg) for r, d in zip(res, vols_dirs)]


def solve_batch(volumes: Sequence, params: TortuosityParams,
                solver_type: DiffusionSolverType = DSOLVER_BICGSTAB) -> List[TauResult]:
    """Many volumes in one call (fast_tau_solve_batch): ``volumes`` is a
    sequence of (mask, dir) pairs, masks 3-D uint8 [z, y, x] of any sizes.
    Every right-hand side advances in the same launches and retires as soon
    as it converges; each result equals solving that volume alone up to the
    summation order of its dot products (the slab depth is chosen for the
    whole launch)."""
    masks, dirs = [], []
    for mask, d in volumes:
        m = _as_mask(mask)
        if m is None:
            raise TypeError("every mask must be a 3-D uint8 array [z, y, x]")
        masks.append(m)
        dirs.append(Dir(d))
    n = len(masks)
    arr = (_native.fast_tau_volume * n)()
    for k, (m, d) in enumerate(zip(masks, dirs)):
        nz, ny, nx = m.shape
        arr[k].mask = m.ctypes.data
        arr[k].nx, arr[k].ny, arr[k].nz, arr[k].dir = nx, ny, nz, int(d)
    p = params.to_c(solver_type)
    res = (_native.fast_tau_result * n)()
    st = _native.lib().fast_tau_solve_batch(arr, n, C.byref(p), res)
    msg = _native.last_error() if st != 0 else ""
    if st not in (0, Status.NO_CONVERGENCE, Status.DIVERGED):
        raise RuntimeError(f"fast_tau_solve_batch: {msg}")
    return _batch_results(res, dirs, msg)


def solve_batch_device(volumes: Sequence, params: TortuosityParams,
                       solver_type: DiffusionSolverType = DSOLVER_BICGSTAB, stream: int = 0) -> List[TauResult]:
    """As solve_batch on device-resident masks: ``volumes`` is a sequence of
    (device pointer, (nz, ny, nx), dir)."""
    n = len(volumes)
    arr = (_native.fast_tau_volume * n)()
    dirs = []
    for k, (ptr, shape, d) in enumerate(volumes):
        nz, ny, nx = shape
        arr[k].mask = int(ptr)
        arr[k].nx, arr[k].ny, arr[k].nz, arr[k].dir = nx, ny, nz, int(d)
        dirs.append(Dir(d))
    p = params.to_c(solver_type)
    res = (_native.fast_tau_result * n)()
    st = _native.lib().fast_tau_solve_batch_device(arr, n, C.byref(p), res, C.c_void_p(stream) if stream else None)
    msg = _native.last_error() if st != 0 else ""
    if st not in (0, Status.NO_CONVERGENCE, Status.DIVERGED):
        raise RuntimeError(f"fast_tau_solve_batch_device: {msg}")
    return _batch_results(res, dirs, msg)
