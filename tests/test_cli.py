"""The `fast tau` command-line drop-in and the .bin volume format.

CPU part: the .bin layout (17-byte header, x-fastest data) round-trips, and
the CLI reports bad arguments and unreadable inputs before any GPU work.
GPU part: rows equal the C-ABI solve of the same volume, the CSV gets the
reference's columns, one header and appended rows, crops behave as the
reference's --sub/--origin."""
import csv
import os
import struct
import subprocess

import numpy as np
import pytest

from fast_gb300 import volume_io

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
COLUMNS = ["ID", "device", "dimx", "dimy", "dimz", "dir", "porosity", "precision", "tau", "tauIter", "tauNU",
           "tauSolver", "tauTime", "tauTolerance"]


@pytest.fixture(scope="module")
def cli(native):
    from fast_gb300 import build
    return build.CLI


def run(cli, *args):
    return subprocess.run([cli, *args], capture_output=True, text=True, timeout=600)


def test_bin_layout_roundtrip(tmp_path):
    m = (np.random.default_rng(1).random((5, 6, 7)) < 0.4).astype(np.uint8) * 255
    p = str(tmp_path / "v.bin")
    volume_io.save_volume_binary(p, m)
    raw = open(p, "rb").read()
    assert len(raw) == 17 + m.size
    assert struct.unpack("<i3i?", raw[:17]) == (2, 7, 6, 5, False)   # UCHAR, x, y, z
    assert raw[17:18] == m[0, 0, :1].tobytes() and raw[-1:] == m[-1, -1, -1:].tobytes()
    v = volume_io.load_volume_binary(p)
    np.testing.assert_array_equal(v.data, m)
    assert v.dim() == (7, 6, 5)
    f = np.arange(24, dtype=np.float32).reshape(2, 3, 4)
    volume_io.save_volume_binary(p, f)
    np.testing.assert_array_equal(volume_io.load_volume_binary(p), f)


def test_cli_errors_without_gpu(cli, tmp_path):
    assert run(cli, "--help").returncode == 0
    assert run(cli, "alpha", "x.bin").returncode == 1
    r = run(cli, "tau", str(tmp_path / "missing.bin"))
    assert r.returncode == 1 and "Couldn't read file" in r.stderr
    p = str(tmp_path / "f.bin")
    volume_io.save_volume_binary(p, np.zeros((2, 2, 2), np.float32))
    r = run(cli, "tau", p)
    assert r.returncode == 1 and "uchar" in r.stderr
    m = str(tmp_path / "m.bin")
    volume_io.save_volume_binary(m, np.zeros((4, 4, 4), np.uint8))
    r = run(cli, "tau", m, "--origin", "1,1,1")          # origin without --sub: empty box
    assert r.returncode == 1 and "Invalid resize" in r.stderr
    r = run(cli, "tau", m, "--aspect", "0.5,0.5,0.5")
    assert r.returncode == 1 and "aspect" in r.stderr
    assert run(cli, "tau", m, "--bogus").returncode == 1


@pytest.mark.gpu
def test_cli_rows_match_c_abi(gpu, cli, tmp_path):
    import fast_gb300 as ft
    from fast_gb300 import volumes
    m = volumes.spheres((30, 26, 34), seed=4, r_min=3.0, solid_fraction=0.5)
    p = str(tmp_path / "vol.bin")
    volume_io.save_volume_binary(p, m)
    out = str(tmp_path / "out.csv")
    r = run(cli, "tau", p, "-d", "pos", "--tol", "8", "--solver", "CG", "-o", out)
    assert r.returncode == 0, r.stderr
    r = run(cli, "tau", p, "-d", "zneg", "--tol", "8", "--solver", "BICGSTAB", "-p", "mixed", "-o", out)
    assert r.returncode == 0, r.stderr
    rows = list(csv.reader(open(out)))
    assert rows[0] == COLUMNS
    assert len(rows) == 5                      # one header, 3 + 1 rows appended
    recs = [dict(zip(COLUMNS, row)) for row in rows[1:]]
    assert [x["dir"] for x in recs] == ["X_POS", "Y_POS", "Z_POS", "Z_NEG"]
    assert [x["precision"] for x in recs] == ["double"] * 3 + ["mixed"]
    phi = float(np.float32((m == 0).mean()))   # the CLI passes porosity rounded to float
    for x, d, solver, prec in zip(recs, [0, 2, 4, 5], ["CG"] * 3 + ["BICGSTAB"], [0, 0, 0, 2]):
        assert (int(x["dimx"]), int(x["dimy"]), int(x["dimz"])) == (34, 26, 30)
        assert x["tauSolver"] == solver and x["device"] == "GPU" and x["tauNU"] == "0"
        assert abs(float(x["tauTolerance"]) - 1e-8) < 1e-20
        assert abs(float(x["porosity"]) - phi) <= 1e-6 * phi
        params = ft.TortuosityParams(dir=ft.Dir(d), tolerance=1e-8, precision=ft.Precision(prec),
                                     porosity=phi, porosity_precomputed=True)
        it = []
        tau = ft.get_tortuosity(m, params, ft.DSOLVER_CG if solver == "CG" else ft.DSOLVER_BICGSTAB,
                                iterations_out=it)
        assert abs(float(x["tau"]) - tau) <= 1e-5 * tau   # the CSV prints 6 significant digits
        assert int(x["tauIter"]) == it[0]


@pytest.mark.gpu
def test_cli_crop_and_stdout(gpu, cli, tmp_path):
    import fast_gb300 as ft
    from fast_gb300 import volumes
    m = volumes.spheres((24, 28, 32), seed=6, r_min=2.5, solid_fraction=0.45)
    p = str(tmp_path / "vol.bin")
    volume_io.save_volume_binary(p, m)
    r = run(cli, "tau", p, "--sub", "20,16,12", "--origin", "4,5,6", "--tol", "8")
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert lines[0].split(",") == COLUMNS and len(lines) == 2
    x = dict(zip(COLUMNS, lines[1].split(",")))
    sub = np.ascontiguousarray(m[6:18, 5:21, 4:24])
    assert (int(x["dimx"]), int(x["dimy"]), int(x["dimz"])) == (20, 16, 12)
    phi = float(np.float32((sub == 0).mean()))
    tau = ft.get_tortuosity(sub, ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-8, porosity=phi,
                                                     porosity_precomputed=True),
                            ft.DSOLVER_CG)
    assert abs(float(x["tau"]) - tau) <= 1e-5 * tau


def test_slice_enumeration_without_gpu(cli, tmp_path):
    # SliceModule.h:66-96: origins stop before origin + size exceeds end, and
    # end defaults to the last voxel index -- a 20^3 volume holds no 20^3
    # sub-volume.  Nothing reaches the GPU on this path.
    m = np.zeros((20, 20, 20), np.uint8)
    p = str(tmp_path / "v.bin")
    volume_io.save_volume_binary(p, m)
    r = run(cli, "slice", p, "--size", "20", "--out", str(tmp_path / "o"))
    assert r.returncode == 0, r.stderr
    assert "Subvolume count 0" in r.stdout and "not big enough" in r.stdout
    r = run(cli, "slice", p, "--size", "0", "--out", str(tmp_path / "o"))
    assert r.returncode == 1


@pytest.mark.gpu
def test_slice_rows(gpu, cli, oracle, tmp_path):
    import ctypes as C
    import fast_gb300 as ft
    nx, ny, nz = 40, 36, 44
    m = np.empty((nz, ny, nx), np.uint8)
    assert gpu.fast_gen_spheres(m.ctypes.data_as(C.c_void_p), nx, ny, nz, 3, 2.0, 4.0, 0.5) == 0
    p = str(tmp_path / "vol.bin")
    volume_io.save_volume_binary(p, m)
    out = tmp_path / "o"
    r = run(cli, "slice", p, "--size", "16", "--stride", "12,10,14", "--out", str(out))
    assert r.returncode == 0, r.stderr
    xs = [x for x in range(0, nx) if x + 16 <= nx - 1][::1]
    origins = [(x, y, z) for x in range(0, nx - 16, 12) for y in range(0, ny - 16, 10) for z in range(0, nz - 16, 14)
               if x + 16 <= nx - 1 and y + 16 <= ny - 1 and z + 16 <= nz - 1]
    assert xs and f"Subvolume count {len(origins)}" in r.stdout
    with open(out / "data.csv") as f:
        header = f.readline().strip().split(",")
    assert header == ["ID", "alpha", "dir", "originx", "originy", "originz", "porosity", "sizex", "sizey", "sizez",
                      "tau"]
    rows = list(csv.DictReader(open(out / "data.csv")))
    assert len(rows) == 3 * len(origins)
    for k, (x, y, z) in enumerate(origins):
        sub = np.ascontiguousarray(m[z:z + 16, y:y + 16, x:x + 16])
        name = f"vol.bin/{x:04d}_{y:04d}_{z:04d}.bin"
        saved = volume_io.load_volume_binary(str(out / name)).data
        np.testing.assert_array_equal(saved, sub)
        phi = float(np.float32((sub == 0).sum() / sub.size))
        for d, dname in enumerate(["X_POS", "Y_POS", "Z_POS"]):
            row = rows[3 * k + d]
            assert row["ID"] == name and row["dir"] == dname
            assert (int(row["originx"]), int(row["originy"]), int(row["originz"])) == (x, y, z)
            assert float(row["porosity"]) == pytest.approx(phi, rel=1e-5)
            ref = oracle.get_tortuosity(sub, dir=2 * d, tol=1e-10)
            if ref["status"] == 0 and ref["tau"] > 0:
                assert float(row["tau"]) == pytest.approx(ref["tau"], rel=1e-3)
        assert float(rows[3 * k]["alpha"]) == pytest.approx(oracle.reactive_area(sub), rel=1e-5)
