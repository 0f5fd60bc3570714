"""Reactive area density (the reference's `fast alpha`): marching-cubes area of
a 0/255 volume's 0.5 iso-surface, over the whole volume and over the pore
space connected to each face, on the GPU through libfasttau.so.

Mirrors fastlib's getReactiveAreaDensity<T>(mask, res, isovalue) and
getReactiveAreaDensityTensor<T>(ccl, res, isovalue)
(fastlib/include/fastlib/volume/VolumeMeasures.h:64-77, VolumeMeasures.cpp:
294-335).  Areas are in the reference's normalized units (axis a scaled by
1/n_a).  ``res`` must be the volume's own dimensions (the only resolution the
reference's `fast alpha` uses); resampling to another grid is not provided.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Tuple

import numpy as np

from . import _native
from .tau import Status, Volume


def _mask_array(mask) -> np.ndarray:
    arr = mask.data if isinstance(mask, Volume) else np.asarray(mask)
    if arr.dtype != np.uint8 or arr.ndim != 3:
        raise TypeError("mask must be a uint8 volume [z, y, x]")
    return np.ascontiguousarray(arr)


def _check_res(arr: np.ndarray, res) -> None:
    if res is None:
        return
    nz, ny, nx = arr.shape
    if tuple(res) not in ((0, 0, 0), (nx, ny, nz)):
        raise NotImplementedError("only res = the volume's dimensions (or 0) is provided")


def _raise(st: int, what: str):
    raise RuntimeError(f"{what} failed ({Status(st).name}): {_native.last_error()}")


def get_reactive_area_density(mask, res=None, isovalue: float = 0.5) -> float:
    """getReactiveAreaDensity<T>(mask, res, isovalue): area of the solid/pore
    interface (voxels != 0 read as 1)."""
    arr = _mask_array(mask)
    _check_res(arr, res)
    nz, ny, nx = arr.shape
    out = C.c_double(0.0)
    st = _native.lib().fast_reactive_area(arr.ctypes.data_as(C.c_void_p), nx, ny, nz, float(isovalue),
                                          C.byref(out))
    if st != Status.OK:
        _raise(st, "reactive area")
    return out.value


def get_reactive_area_density_tensor(mask, res=None, isovalue: float = 0.5,
                                     with_solid: bool = False):
    """getVolumeCCL(mask, 255) + getReactiveAreaDensityTensor<T>: six areas in
    Dir order, each of the pore components touching that face.  With
    ``with_solid`` the whole-volume area of get_reactive_area_density, from
    the same pass, is returned too: (tensor, area)."""
    arr = _mask_array(mask)
    _check_res(arr, res)
    nz, ny, nx = arr.shape
    tensor = (C.c_double * 6)()
    solid = C.c_double(0.0)
    st = _native.lib().fast_reactive_area_tensor(arr.ctypes.data_as(C.c_void_p), nx, ny, nz, float(isovalue),
                                                 tensor, C.byref(solid))
    if st != Status.OK:
        _raise(st, "reactive area tensor")
    t = [float(v) for v in tensor]
    return (t, solid.value) if with_solid else t


def get_reactive_area_density_tensor_device(d_mask, shape: Tuple[int, int, int], isovalue: float = 0.5,
                                            stream: Optional[int] = None) -> Tuple[List[float], float]:
    """The tensor on a device-resident mask (a CUDA pointer as int, shape
    (nz, ny, nx)); returns (tensor, area)."""
    nz, ny, nx = shape
    tensor = (C.c_double * 6)()
    solid = C.c_double(0.0)
    st = _native.lib().fast_reactive_area_tensor_device(C.c_void_p(d_mask), nx, ny, nz, float(isovalue), tensor,
                                                        C.byref(solid), C.c_void_p(stream or 0))
    if st != Status.OK:
        _raise(st, "reactive area tensor")
    return [float(v) for v in tensor], solid.value


__all__ = ["get_reactive_area_density", "get_reactive_area_density_tensor",
           "get_reactive_area_density_tensor_device"]
