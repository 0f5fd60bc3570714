"""Golden assembly records made by the reference's own code.

oracle/Makefile's `ref` target compiles getSystemTopKernel<T>
(fastlib/src/cuda/Diffusion.cuh:54-148), the reference's per-voxel rule for
the 7 stored coefficients, the right-hand side and the initial guess, for the
host, from the reference's source (the reference tree must be present, as in
the build container).  This script runs it on seeded volumes in every
direction, in FP64 and FP32, and stores the SHA-256 of each output array in
ref_assembly.json.  tests/test_oracle.py checks the oracle's restated
assembly against these records on any host, and against the built library
itself where it exists.

Usage:  python tests/golden/make_ref_golden.py
"""
import ctypes as C
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

REF_SO = os.path.join(ROOT, "oracle", "_ref", "libref_assembly.so")
D0 = float(np.float32(1.0))
D1 = float(np.float32(0.001))


def cases():
    """(name, mask) pairs: generator volumes and random phase fields,
    including one-voxel and one-plane axes."""
    from oracle import oracle as O
    out = [("spheres_12x14x16", O.gen_spheres((16, 14, 12), 1, 3.0, 3.0, 0.5)),
           ("spheres_25x17x9", O.gen_spheres((9, 17, 25), 3, 2.0, 2.0, 0.4)),
           ("ellipsoids_16", O.gen_ellipsoids((16, 16, 16), 4, 5.0, 0.35, 0.55))]
    for shape, seed in (((7, 9, 11), 5), ((1, 6, 5), 6), ((4, 1, 3), 7), ((1, 1, 8), 8), ((3, 2, 1), 9)):
        out.append((f"random_{shape[2]}x{shape[1]}x{shape[0]}",
                    ((np.random.default_rng(seed).random(shape) < 0.5) * 255).astype(np.uint8)))
    return out


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ref_lib():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref"], check=True)
    L = C.CDLL(REF_SO)
    P, i64 = C.c_void_p, C.c_int64
    for sfx in ("f64", "f32"):
        getattr(L, f"ref_assemble_{sfx}").argtypes = [P, i64, i64, i64, C.c_int, C.c_double, C.c_double,
                                                       C.c_float, P, P, P]
        getattr(L, f"ref_assemble_{sfx}").restype = C.c_int
    return L


def ref_assemble(L, mask, d, dtype):
    nz, ny, nx = mask.shape
    N = mask.size
    A = np.empty((7, N), dtype=dtype)
    b = np.empty(N, dtype=dtype)
    x0 = np.empty(N, dtype=dtype)
    cell = np.float32(1.0) / np.float32(max(nx, ny, nz))
    sfx = "f64" if dtype == np.float64 else "f32"
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    st = getattr(L, f"ref_assemble_{sfx}")(ptr(mask), nx, ny, nz, d, D0, D1, float(cell), ptr(A), ptr(b), ptr(x0))
    assert st == 0
    return A, b, x0


def main():
    L = ref_lib()
    recs = []
    for name, m in cases():
        e = {"name": name, "shape": list(m.shape), "mask_sha256": sha(m), "dirs": {}}
        if name.startswith("random"):
            e["volume"] = m.reshape(-1).tolist()
        for d in range(6):
            e["dirs"][str(d)] = {}
            for dt, tag in ((np.float64, "f64"), (np.float32, "f32")):
                A, b, x0 = ref_assemble(L, m, d, dt)
                e["dirs"][str(d)][tag] = {"A": sha(A), "b": sha(b), "x0": sha(x0)}
        recs.append(e)
    with open(os.path.join(HERE, "ref_assembly.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_ref_golden.py",
                   "reference_code": "getSystemTopKernel<T>, fastlib/src/cuda/Diffusion.cuh:54-148",
                   "d0": D0, "d1": D1, "cases": recs}, f, indent=1)


if __name__ == "__main__":
    main()
