"""The C++ front end (include/fasttau.hpp) with fastlib's signatures:
fast::Volume, fast::TortuosityParams, fast::getTortuosity<T> and
fast::getPorosity<T> (fastlib/include/fastlib/volume/VolumeMeasures.h:15-61).

A small program (tests/cpp/shim_check.cpp) is compiled against the header
and linked to libfasttau.so: on the CPU the test checks that it builds; on
the GPU it runs getTortuosity<double> and <float> with the concentration
output and compares tau, the iteration count, porosity and the field with
the oracle (FP64 at tol 1e-10: CG within 1e-9 with iterations within 2,
BiCGSTAB within 1e-8; FP32 at tol 1e-5 within 1e-4 of the float oracle)."""
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _build(native, out_dir):
    from fast_gb300 import build
    exe = os.path.join(out_dir, "shim_check")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "cpp", "shim_check.cpp"), "-o", exe, build.LIB, "-Wl,-rpath," + os.path.dirname(build.LIB)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles(native, tmp_path):
    assert os.path.exists(_build(native, str(tmp_path)))


@pytest.mark.gpu
@pytest.mark.parametrize("d,solver", [(0, 1), (3, 1), (4, 0)])
def test_shim_matches_oracle(gpu, oracle, tmp_path, d, solver):
    from fast_gb300 import volume_io, volumes
    exe = _build(gpu, str(tmp_path))
    m = volumes.spheres((22, 26, 30), seed=40 + d, r_min=3.0, solid_fraction=0.5)
    path = str(tmp_path / "v.bin")
    volume_io.save_volume_binary(path, m)
    tol = 1e-10
    r = subprocess.run([exe, path, str(d), str(solver), str(tol), "1e-5"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = {ln.split()[0]: ln.split()[1:] for ln in r.stdout.splitlines()}
    phi = (m == 0).sum() / m.size
    ref = oracle.get_tortuosity(m, dir=d, solver=solver, tol=tol, return_conc=True)
    tau, por, iters, csum, c0 = (float(rows["double"][0]), float(rows["double"][1]), int(rows["double"][2]),
                                 float(rows["double"][3]), float(rows["double"][4]))
    assert abs(por - phi) < 1e-15
    lim = 1e-9 if solver == 1 else 1e-8
    assert abs(tau - ref["tau"]) / ref["tau"] <= lim
    if solver == 1:
        assert abs(iters - ref["iters"]) <= 2
    assert abs(csum - float(ref["conc"].sum())) <= 1e-7 * m.size
    assert abs(c0 - float(ref["conc"].reshape(-1)[0])) <= 1e-8
    ref32 = oracle.get_tortuosity(m, dir=d, solver=solver, tol=1e-5, dtype=np.float32)
    assert ref32["status"] == 0
    tau32 = float(rows["float"][0])
    assert abs(tau32 - ref32["tau"]) / ref32["tau"] <= 1e-4
