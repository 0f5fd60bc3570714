"""Bounds-checked build (FAST_TAU_BOUNDS_CHECK=1): every plain global load and
store of the solver kernels checks its index, records the first failing site
in the right-hand side's scalars and skips the access; the call then fails
with "bounds check".  This test builds that variant of the library, runs the
awkward shapes (one-voxel axes, a one-plane primary axis, sizes that are not
tile multiples) in every direction, precision and solver, slab depths of 3
and 64 planes, and batches of mixed sizes through it in a child process, and requires that no access was
out of range and the results equal the regular build's."""
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

SCRIPT = r"""
import json, sys
import numpy as np
sys.path.insert(0, %(root)r)
import fast_gb300 as ft
from fast_gb300 import volumes
out = []
shapes = [(1, 1, 1), (1, 5, 1), (7, 1, 1), (1, 1, 9), (3, 17, 2), (2, 3, 70), (33, 5, 65), (20, 70, 19)]
for s in shapes:
    m = volumes.spheres(s, 3, 1.0, 2.0, 0.3) if min(s) > 2 else np.zeros(s, np.uint8)
    for d in range(6):
        for prec in (ft.Precision.F64, ft.Precision.F32, ft.Precision.MIXED):
            for solver in (ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB):
                p = ft.TortuosityParams(dir=ft.Dir(d), tolerance=1e-6, precision=prec)
                try:
                    tau = ft.get_tortuosity(m, p, solver)
                    err = ""
                except Exception as e:
                    tau, err = 0.0, str(e)
                out.append([list(s), d, int(prec), int(solver), tau, err])
import os
for zc in ("3", "64"):
    os.environ["FAST_TAU_ZC"] = zc
    for s in [(70, 9, 33), (130, 20, 17)]:
        m = volumes.spheres(s, 3, 1.0, 2.0, 0.3)
        for d in (0, 5):
            for prec in (ft.Precision.F64, ft.Precision.MIXED):
                for solver in (ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB):
                    p = ft.TortuosityParams(dir=ft.Dir(d), tolerance=1e-6, precision=prec)
                    try:
                        tau = ft.get_tortuosity(m, p, solver)
                        err = ""
                    except Exception as e:
                        tau, err = 0.0, str(e)
                    out.append(["zc" + zc, list(s), d, int(prec), int(solver), tau, err])
os.environ.pop("FAST_TAU_ZC", None)
vols = [volumes.spheres(s, 5, 1.0, 2.0, 0.35) for s in [(9, 33, 17), (40, 8, 3), (16, 16, 16)]]
p = ft.TortuosityParams(tolerance=1e-6, precision=ft.Precision.MIXED)
res = ft.solve_batch(list(zip(vols, [ft.Dir.X_POS, ft.Dir.Y_NEG, ft.Dir.Z_POS])), p, ft.DSOLVER_CG)
out.append(["batch", [r.tau for r in res], [int(r.status) for r in res]])
print(json.dumps(out))
"""


@pytest.fixture(scope="module")
def checked_lib(tmp_path_factory):
    from fast_gb300 import build as b
    out = str(tmp_path_factory.mktemp("bounds"))
    code = (
        "import os, sys; sys.path.insert(0, %r)\n"
        "import fast_gb300.build as b\n"
        "b.OUT = %r; b.LIB = os.path.join(b.OUT, 'libfasttau.so'); b.CLI = os.path.join(b.OUT, 'fast')\n"
        "print(b.build(force=True))\n" % (ROOT, out))
    env = dict(os.environ, FAST_TAU_NVCC_FLAGS="-DFAST_TAU_BOUNDS_CHECK=1")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=1800)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout.strip().splitlines()[-1]


def _run(lib=None):
    env = dict(os.environ)
    if lib:
        env["FAST_TAU_LIB"] = lib
    r = subprocess.run([sys.executable, "-c", SCRIPT % {"root": ROOT}], capture_output=True, text=True, env=env,
                       timeout=1800)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "bounds check" not in r.stderr, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.gpu
def test_no_out_of_range_access(gpu, checked_lib):
    checked = _run(checked_lib)
    plain = _run()
    assert len(checked) == len(plain)
    for a, b in zip(checked, plain):
        assert "bounds check" not in json.dumps(a), a
        assert a == b, (a, b)
