"""Connected components of a phase volume on the GPU: the mirror of fastlib's
VolumeCCL / getVolumeCCL (fastlib/include/fastlib/volume/VolumeSegmentation.h,
fastlib/src/volume/VolumeSegmentation.cpp:9-90), served by libfasttau.so's
fast_ccl_label, fast_ccl_label_device and fast_ccl_boundary_device.

Numbering is the reference's: 0 = background, components 1..K ordered by
their smallest linear index (x fastest), num_labels = K + 1; the boundary
mask has one row per Dir (X_POS = the x = nx-1 face) plus a seventh row, the
AND of the six (labels touching every face)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _native
from .tau import Dir, _as_mask

_FIRST_GUESS_LABELS = 1 << 20
_BAD_ARG = 8


def _raise(fn: str, st: int):
    raise RuntimeError(f"{fn} failed ({st}): {_native.last_error()}")


@dataclass
class VolumeCCL:
    num_labels: int                       # includes label 0 (background)
    labels: Optional[np.ndarray]          # uint32 [nz, ny, nx] (host API)
    boundary_label_mask: np.ndarray       # uint8 [7, num_labels]
    background: int = 255

    def get_dir_mask(self, begin: Dir, end: Optional[Dir] = None) -> np.ndarray:
        """getDirMask(dir): labels touching face `dir`; getDirMask(begin,
        end): labels touching both faces (VolumeSegmentation.cpp:9-24)."""
        if end is None:
            return self.boundary_label_mask[int(begin)]
        return (self.boundary_label_mask[int(begin)] & self.boundary_label_mask[int(end)]).astype(np.uint8)


def get_volume_ccl(mask, background: int = 255) -> VolumeCCL:
    """getVolumeCCL(mask, background) on a host mask: labels and the
    boundary rows in one GPU pass (a second one only when the volume has
    more than 2^20 components and the first boundary buffer was too small)."""
    m = _as_mask(mask)
    if m is None:
        raise TypeError("mask must be a 3-D uint8 array [z, y, x]")
    nz, ny, nx = m.shape
    L = _native.lib()
    labels = np.empty(m.shape, dtype=np.uint32)
    n = C.c_uint32(0)
    cap_labels = min(m.size // 2 + 2, _FIRST_GUESS_LABELS)
    for _ in range(2):
        bnd = np.zeros(7 * cap_labels, dtype=np.uint8)
        st = L.fast_ccl_label(m.ctypes.data_as(C.c_void_p), nx, ny, nz, int(background),
                              labels.ctypes.data_as(C.c_void_p), C.byref(n), bnd.ctypes.data_as(C.c_void_p),
                              bnd.nbytes)
        if st == _BAD_ARG and n.value > cap_labels:
            cap_labels = int(n.value)
            continue
        if st != 0:
            _raise("fast_ccl_label", st)
        break
    k = int(n.value)
    return VolumeCCL(k, labels, bnd[:7 * k].reshape(7, k).copy(), int(background))


def get_volume_ccl_device(d_mask_ptr: int, shape, d_labels_ptr: int, background: int = 255,
                          boundary: bool = True, stream: Optional[int] = None) -> VolumeCCL:
    """getVolumeCCL(const CUDA_Volume&, background) on a DEVICE mask (a
    pointer such as ``tensor.data_ptr()``), labels into caller-owned device
    memory (uint32, same shape); the returned VolumeCCL holds no host labels."""
    nz, ny, nx = shape
    L = _native.lib()
    n = C.c_uint32(0)
    sp = C.c_void_p(stream) if stream else None
    st = L.fast_ccl_label_device(C.c_void_p(d_mask_ptr), nx, ny, nz, int(background), C.c_void_p(d_labels_ptr),
                                 C.byref(n), None, 0, sp)
    if st != 0:
        _raise("fast_ccl_label_device", st)
    k = int(n.value)
    bnd = np.zeros((7, k), dtype=np.uint8)
    if boundary:
        st = L.fast_ccl_boundary_device(C.c_void_p(d_labels_ptr), nx, ny, nz, k, bnd.ctypes.data_as(C.c_void_p), sp)
        if st != 0:
            _raise("fast_ccl_boundary_device", st)
    return VolumeCCL(k, None, bnd, int(background))


def generate_boundary_connected_volume(ccl: VolumeCCL, dir: Dir, invert_mask: bool = False) -> np.ndarray:
    """generateBoundaryConnectedVolume (VolumeSegmentation.cpp:66-88) on the
    host labels: 255 where the voxel's label touches face `dir` (inverted:
    does not; label 0 is never inverted), else 0."""
    if ccl.labels is None:
        raise ValueError("needs the host labels of get_volume_ccl")
    sel = ccl.get_dir_mask(dir).astype(bool).copy()
    if invert_mask:
        sel[1:] = ~sel[1:]
    return np.where(sel[ccl.labels], np.uint8(255), np.uint8(0))


__all__ = ["VolumeCCL", "get_volume_ccl", "get_volume_ccl_device", "generate_boundary_connected_volume"]
