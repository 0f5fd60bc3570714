"""Seeded synthetic microstructures (255 = solid, 0 = pore), generated by
libfasttau.so's host code so the same seed gives the same bytes on every host.

``spheres`` / ``ellipsoids`` return uint8 arrays indexed [z, y, x].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native


def spheres(shape, seed: int, r_min: float, r_max: float = None, solid_fraction: float = 0.5) -> np.ndarray:
    """Overlapping solid spheres (radius uniform in [r_min, r_max] voxels)
    added until the solid fraction reaches ``solid_fraction``."""
    nz, ny, nx = shape
    out = np.empty((nz, ny, nx), dtype=np.uint8)
    r_max = r_min if r_max is None else r_max
    st = _native.lib().fast_gen_spheres(out.ctypes.data_as(C.c_void_p), nx, ny, nz, seed, r_min, r_max,
                                        solid_fraction)
    if st != 0:
        raise ValueError(f"fast_gen_spheres failed with status {st}")
    return out


def ellipsoids(shape, seed: int, semi_major: float, aspect: float, solid_fraction: float) -> np.ndarray:
    """Randomly oriented solid ellipsoids with semi-axes (a, a*aspect,
    a*aspect), overlap allowed, added until the solid fraction is reached."""
    nz, ny, nx = shape
    out = np.empty((nz, ny, nx), dtype=np.uint8)
    st = _native.lib().fast_gen_ellipsoids(out.ctypes.data_as(C.c_void_p), nx, ny, nz, seed, semi_major, aspect,
                                           solid_fraction)
    if st != 0:
        raise ValueError(f"fast_gen_ellipsoids failed with status {st}")
    return out
