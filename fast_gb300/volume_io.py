"""Volume files of the reference's `.bin` format (fastlib/src/volume/
VolumeIO.cpp:256-305 saveVolumeBinary / loadVolumeBinary): a 17-byte header
-- int32 PrimitiveType, int32 x 3 dimensions (x, y, z), one bool byte the
reference no longer uses -- then the raw voxels, x fastest, little endian.
Arrays here are [z, y, x] (x fastest in memory), as everywhere in the
package; the tortuosity path reads PrimitiveType UCHAR (2) volumes.  Folders
of TIFF slices (loadTiffFolder) are read by load_tiff_folder."""
from __future__ import annotations

import os
import struct

import numpy as np

from .tau import Volume

# PrimitiveType (fastlib/include/fastlib/utility/PrimitiveTypes.h:11-24):
# numpy element type and components per voxel.
PRIMITIVE_TYPES = {
    0: (np.float32, 1),   # TYPE_FLOAT
    1: (np.int8, 1),      # TYPE_CHAR
    2: (np.uint8, 1),     # TYPE_UCHAR
    3: (np.int32, 1),     # TYPE_INT
    4: (np.uint32, 1),    # TYPE_UINT
    5: (np.uint64, 1),    # TYPE_UINT64
    6: (np.float32, 3),   # TYPE_FLOAT3
    7: (np.float32, 4),   # TYPE_FLOAT4
    8: (np.float64, 1),   # TYPE_DOUBLE
    9: (np.uint8, 3),     # TYPE_UCHAR3
    10: (np.uint8, 4),    # TYPE_UCHAR4
}
HEADER = struct.Struct("<i3i?")  # 17 bytes


def _type_of(arr: np.ndarray) -> int:
    comps = 1 if arr.ndim == 3 else arr.shape[-1]
    for code, (dt, c) in PRIMITIVE_TYPES.items():
        if np.dtype(dt) == arr.dtype and c == comps:
            return code
    raise TypeError(f"no PrimitiveType for {arr.dtype} x {comps}")


def save_volume_binary(path: str, data) -> None:
    """saveVolumeBinary: `data` is a Volume or an array [z, y, x] (or
    [z, y, x, components] for the vector types)."""
    arr = data.data if isinstance(data, Volume) else np.asarray(data)
    if arr.ndim not in (3, 4):
        raise ValueError("volume must be [z, y, x] or [z, y, x, c]")
    nz, ny, nx = arr.shape[:3]
    with open(path, "wb") as f:
        f.write(HEADER.pack(_type_of(arr), nx, ny, nz, False))
        f.write(np.ascontiguousarray(arr).tobytes())


def load_volume_binary(path: str):
    """loadVolumeBinary: returns a Volume for UCHAR volumes, else the array
    ([z, y, x] or [z, y, x, components])."""
    with open(path, "rb") as f:
        head = f.read(HEADER.size)
        if len(head) != HEADER.size:
            raise ValueError("Couldn't read file: truncated header")
        code, nx, ny, nz, _ = HEADER.unpack(head)
        if code not in PRIMITIVE_TYPES or min(nx, ny, nz) <= 0:
            raise ValueError(f"bad .bin header (type {code}, dims {nx} {ny} {nz})")
        dt, comps = PRIMITIVE_TYPES[code]
        count = nx * ny * nz * comps
        arr = np.fromfile(f, dtype=dt, count=count)
    if arr.size != count:
        raise ValueError("Couldn't read file: truncated data")
    arr = arr.reshape((nz, ny, nx) if comps == 1 else (nz, ny, nx, comps))
    return Volume(arr) if code == Volume.TYPE_UCHAR else arr


def load_tiff_folder(folder: str, binarize: bool = False, threshold: float = 1.0) -> Volume:
    """loadTiffFolder (VolumeIO.cpp:197-254): the folder's *.tif / *.tiff
    slices, in byte-wise name order, stacked along z into a uint8 Volume
    [z, y, x].  The slices are decoded by libfasttau's TIFF reader
    (fast_tiff_folder_info / fast_tiff_folder_read).  ``binarize=True``
    applies Volume::binarize(threshold) on the GPU afterwards, which is what
    `fast tau` does with a folder input (VolumeIOModule.h:57-63)."""
    import ctypes as C

    from . import _native
    from .tau import Status

    L = _native.lib()
    path = os.fsencode(folder)
    nx, ny, nz = C.c_int64(), C.c_int64(), C.c_int64()
    st = L.fast_tiff_folder_info(path, C.byref(nx), C.byref(ny), C.byref(nz))
    if st != Status.OK:
        raise OSError(f"Failed to load {folder} ({Status(st).name}): {_native.last_error()}")
    arr = np.empty((nz.value, ny.value, nx.value), np.uint8)
    st = L.fast_tiff_folder_read(path, arr.ctypes.data_as(C.c_void_p), arr.nbytes)
    if st != Status.OK:
        raise OSError(f"Failed to load {folder} ({Status(st).name}): {_native.last_error()}")
    vol = Volume(arr)
    if binarize:
        vol.binarize(threshold)
    return vol


__all__ = ["load_volume_binary", "save_volume_binary", "load_tiff_folder", "PRIMITIVE_TYPES"]
