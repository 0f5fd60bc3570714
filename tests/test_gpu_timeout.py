"""The bounded device-side wait and its failure path (FAST_TIMEOUT).

Every mbarrier wait of the solver sweeps gives up after a time limit; the
block then drains the tile loads it still has in flight, marks its
right-hand side FAULT and returns, and the call reports FAST_TIMEOUT with the
context still usable.  This test builds a variant of the library with test
hooks and a 50 ms limit (FAST_TAU_TEST_HOOKS=1, FAST_TAU_WAIT_LIMIT_NS), arms
the hook for one direction (FAST_TAU_TEST_WITHHOLD = 1 + direction: the first
sweep of that right-hand side does not issue the tile loads of one plane in
one block, so the wait for them runs out), and checks, in a child process:

  * FP64 CG, three directions in one call: the armed direction returns
    FAST_TIMEOUT, the other two return the same tau as an unarmed call;
  * MIXED BiCGSTAB (the first sweep is the replacement kernel that walks
    tiles with a resident grid): the armed call returns FAST_TIMEOUT;
  * the next call in the same process succeeds with the unarmed results;
  * with the device's free memory faked small (FAST_TAU_TEST_FREE_BYTES), a
    solve fails with FAST_NOMEM before any device work, as the reference's
    fit check makes it fail.

No wait is unbounded and nothing traps: the failure is a status.
"""
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

SCRIPT = r"""
import ctypes as C, json, os, sys
sys.path.insert(0, %(root)r)
import fast_gb300 as ft
from fast_gb300 import _native, volumes
L = _native.lib()
m = volumes.spheres((40, 36, 44), seed=8, r_min=3.0, solid_fraction=0.5)
nz, ny, nx = m.shape

def solve(dirs, prec, solver, arm=None):
    if arm is not None:
        os.environ["FAST_TAU_TEST_WITHHOLD"] = str(arm + 1)
    else:
        os.environ.pop("FAST_TAU_TEST_WITHHOLD", None)
    p = ft.TortuosityParams(tolerance=1e-8, precision=prec).to_c(solver)
    arr = (C.c_int32 * len(dirs))(*dirs)
    res = (_native.fast_tau_result * len(dirs))()
    st = L.fast_tau_solve_dirs(m.ctypes.data_as(C.c_void_p), nx, ny, nz, C.byref(p), len(dirs), arr, res)
    return [int(st), [[int(r.status), r.tau] for r in res]]

out = {}
os.environ["FAST_TAU_TEST_FREE_BYTES"] = "1000000"
out["nomem"] = solve([0], ft.Precision.F64, ft.DSOLVER_CG)
out["nomem_msg"] = _native.last_error()
os.environ.pop("FAST_TAU_TEST_FREE_BYTES")
out["f64_armed"] = solve([0, 2, 4], ft.Precision.F64, ft.DSOLVER_CG, arm=2)
out["f64_after"] = solve([0, 2, 4], ft.Precision.F64, ft.DSOLVER_CG)
out["mixed_armed"] = solve([1], ft.Precision.MIXED, ft.DSOLVER_BICGSTAB, arm=1)
out["mixed_after"] = solve([1], ft.Precision.MIXED, ft.DSOLVER_BICGSTAB)
out["mixed_plain"] = solve([1], ft.Precision.MIXED, ft.DSOLVER_BICGSTAB)
print(json.dumps(out))
"""

FAST_OK, FAST_NOMEM, FAST_TIMEOUT = 0, 3, 7


@pytest.fixture(scope="module")
def hooked_lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("hooks"))
    code = (
        "import os, sys; sys.path.insert(0, %r)\n"
        "import fast_gb300.build as b\n"
        "b.OUT = %r; b.LIB = os.path.join(b.OUT, 'libfasttau.so'); b.CLI = os.path.join(b.OUT, 'fast')\n"
        "print(b.build(force=True))\n" % (ROOT, out))
    env = dict(os.environ,
               FAST_TAU_NVCC_FLAGS="-DFAST_TAU_TEST_HOOKS=1 -DFAST_TAU_WAIT_LIMIT_NS=50000000ull")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=1800)
    assert r.returncode == 0, r.stderr[-2000:]
    return r.stdout.strip().splitlines()[-1]


@pytest.mark.gpu
def test_withheld_tile_load_times_out_and_context_recovers(gpu, hooked_lib):
    env = dict(os.environ, FAST_TAU_LIB=hooked_lib)
    env.pop("FAST_TAU_TEST_WITHHOLD", None)
    r = subprocess.run([sys.executable, "-c", SCRIPT % {"root": ROOT}], capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])

    # the reference's fit check (VolumeMeasures.cpp:104-125): a solve that
    # does not fit fails with FAST_NOMEM before touching the device
    assert out["nomem"][0] == FAST_NOMEM and "will not fit" in out["nomem_msg"]

    st, res = out["f64_armed"]
    st_after, res_after = out["f64_after"]
    assert st == FAST_TIMEOUT
    assert res[1][0] == FAST_TIMEOUT and res[1][1] == 0.0
    assert st_after == FAST_OK and all(s == FAST_OK for s, _ in res_after)
    # the directions that were not armed are untouched by the failed one
    assert res[0] == res_after[0] and res[2] == res_after[2]

    st, res = out["mixed_armed"]
    assert st == FAST_TIMEOUT and res[0][0] == FAST_TIMEOUT
    st_after, res_after = out["mixed_after"]
    assert st_after == FAST_OK and res_after[0][0] == FAST_OK
    assert res_after == out["mixed_plain"][1]
