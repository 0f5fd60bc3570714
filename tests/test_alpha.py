"""Reactive area density (`fast alpha`: getReactiveAreaDensity and its
per-face tensor, VolumeMeasures.cpp:294-335; marching cubes in
VolumeSurface.cu:143-262).

CPU part: the oracle's known answers -- an axis-aligned interface has area
1.0 in normalized units whatever the triangulation, empty and full volumes
have none, a voxelised sphere comes out within a few percent of 4 pi R^2 --
and its per-face tensor equals the area of the face-connected pore space
built by hand.  GPU part: the engine's one-pass seven-field area equals the
oracle on random and packed volumes of awkward sizes and isovalues (per-cell
arithmetic is the same float sequence; only the order of the double sums
differs), the device entry equals the host one, non-binary masks are
refused, and `fast alpha` writes the reference's rows and columns."""
import csv
import ctypes as C
import math
import subprocess

import numpy as np
import pytest

from fast_gb300 import Status, volume_io

X_POS, X_NEG, Y_POS, Y_NEG, Z_POS, Z_NEG = range(6)


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.mark.parametrize("shape", [(20, 24, 28), (7, 33, 9), (1, 5, 40)])
def test_plane_area_is_one(oracle, shape):
    nz, ny, nx = shape
    for axis, n in ((2, nx), (1, ny), (0, nz)):
        if n < 2:
            continue
        for cut in sorted({1, n // 2, n - 1}):
            m = np.zeros(shape, np.uint8)
            sl = [slice(None)] * 3
            sl[axis] = slice(0, cut)
            m[tuple(sl)] = 255
            assert abs(oracle.reactive_area(m) - 1.0) < 1e-5, (axis, cut)


def test_empty_full_and_table(oracle):
    assert oracle.reactive_area(np.zeros((9, 10, 11), np.uint8)) == 0.0
    assert oracle.reactive_area(np.full((9, 10, 11), 255, np.uint8)) == 0.0
    counts = [oracle.lib().oracle_mc_ntri(c) for c in range(256)]
    assert counts[0] == counts[255] == 0
    assert max(counts) == 5 and min(counts[1:255]) >= 1
    # A single below corner cuts three edges: one triangle.
    assert all(counts[1 << c] == 1 and counts[255 ^ (1 << c)] == 1 for c in range(8))


def test_sphere_area(oracle):
    n, r = 64, 20.0
    z, y, x = np.mgrid[:n, :n, :n]
    m = ((((x - 31.5) ** 2 + (y - 31.5) ** 2 + (z - 31.5) ** 2) < r * r) * 255).astype(np.uint8)
    a = oracle.reactive_area(m) * n * n
    assert 1.0 <= a / (4 * math.pi * r * r) <= 1.05


def test_tensor_by_hand(oracle):
    # A pore channel along x (touches X faces only), an isolated pore cube,
    # solid elsewhere; pores are 0, solid 255.
    m = np.full((16, 18, 20), 255, np.uint8)
    m[5:9, 6:10, :] = 0
    m[11:14, 12:15, 4:8] = 0
    t = oracle.reactive_area_tensor(m)
    chan = np.zeros_like(m)
    chan[5:9, 6:10, :] = 1
    a = oracle.area_field(chan)
    assert a > 0
    assert t[X_POS] == pytest.approx(a, rel=1e-12) and t[X_NEG] == pytest.approx(a, rel=1e-12)
    assert t[Y_POS] == t[Y_NEG] == t[Z_POS] == t[Z_NEG] == 0.0


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

def _area(gpu, m, iso=0.5):
    nz, ny, nx = m.shape
    out = C.c_double()
    st = gpu.fast_reactive_area(m.ctypes.data_as(C.c_void_p), nx, ny, nz, iso, C.byref(out))
    assert st == Status.OK, gpu.fast_last_error()
    return out.value


def _tensor(gpu, m, iso=0.5):
    nz, ny, nx = m.shape
    t = (C.c_double * 6)()
    solid = C.c_double()
    st = gpu.fast_reactive_area_tensor(m.ctypes.data_as(C.c_void_p), nx, ny, nz, iso, t, C.byref(solid))
    assert st == Status.OK, gpu.fast_last_error()
    return list(t), solid.value


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(1, 1, 1), (1, 6, 45), (3, 9, 33), (17, 31, 40), (40, 8, 64), (65, 66, 67)])
@pytest.mark.parametrize("iso", [0.5, 0.3, 0.8, 1.0])
def test_area_parity_random(gpu, oracle, shape, iso):
    rng = np.random.default_rng(sum(shape))
    m = ((rng.random(shape) < 0.45) * 255).astype(np.uint8)
    got, want = _area(gpu, m, iso), oracle.reactive_area(m, iso)
    assert rel(got, want) <= 1e-11 or abs(got - want) < 1e-14


@pytest.mark.gpu
@pytest.mark.parametrize("shape,solid", [((48, 48, 48), 0.6), ((37, 50, 29), 0.5), ((64, 24, 96), 0.7)])
def test_tensor_parity_packed(gpu, oracle, shape, solid):
    nz, ny, nx = shape
    m = np.empty(shape, np.uint8)
    st = gpu.fast_gen_spheres(m.ctypes.data_as(C.c_void_p), nx, ny, nz, 11, 3.0, 6.0, solid)
    assert st == Status.OK
    t, area = _tensor(gpu, m)
    want_t = oracle.reactive_area_tensor(m)
    want_a = oracle.reactive_area(m)
    assert rel(area, want_a) <= 1e-11
    for d in range(6):
        assert rel(t[d], want_t[d]) <= 1e-11 or abs(t[d] - want_t[d]) < 1e-14, d
    assert any(v > 0 for v in t)
    # Repeatable to the last bit.
    assert _tensor(gpu, m) == (t, area)
    assert _area(gpu, m) == area


@pytest.mark.gpu
def test_device_entries_and_refusals(gpu, oracle):
    import torch
    from fast_gb300 import alpha
    rng = np.random.default_rng(3)
    m = ((rng.random((30, 26, 34)) < 0.5) * 255).astype(np.uint8)
    d = torch.from_numpy(m).cuda()
    s = torch.cuda.current_stream().cuda_stream
    t_dev, a_dev = alpha.get_reactive_area_density_tensor_device(d.data_ptr(), m.shape, 0.5, s)
    t_host, a_host = alpha.get_reactive_area_density_tensor(m, with_solid=True)
    assert (t_dev, a_dev) == (t_host, a_host)
    out = C.c_double()
    st = gpu.fast_reactive_area_device(C.c_void_p(d.data_ptr()), 34, 26, 30, 0.5, C.byref(out), C.c_void_p(s))
    assert st == Status.OK and out.value == a_host == alpha.get_reactive_area_density(m)
    bad = m.copy()
    bad[3, 4, 5] = 7
    nz, ny, nx = bad.shape
    st = gpu.fast_reactive_area(bad.ctypes.data_as(C.c_void_p), nx, ny, nz, 0.5, C.byref(out))
    assert st == Status.BAD_TYPE
    assert gpu.fast_reactive_area(bad.ctypes.data_as(C.c_void_p), 0, ny, nz, 0.5, C.byref(out)) == Status.BAD_ARG
    with pytest.raises(NotImplementedError):
        alpha.get_reactive_area_density(m, res=(10, 10, 10))


@pytest.mark.gpu
def test_cli_alpha(gpu, oracle, tmp_path):
    from fast_gb300 import build
    m = np.empty((24, 28, 32), np.uint8)
    assert gpu.fast_gen_spheres(m.ctypes.data_as(C.c_void_p), 32, 28, 24, 5, 3.0, 5.0, 0.55) == Status.OK
    p = str(tmp_path / "v.bin")
    volume_io.save_volume_binary(p, m)
    out = str(tmp_path / "a.csv")
    r = subprocess.run([build.CLI, "alpha", p, "-d", "all", "-o", out], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    with open(out) as f:
        header = f.readline().strip().split(",")
    assert header == ["ID", "dimx", "dimy", "dimz", "dir", "porosity", "rad", "radTime"]
    rows = list(csv.DictReader(open(out)))
    assert [r["dir"] for r in rows] == ["X_POS", "X_NEG", "Y_POS", "Y_NEG", "Z_POS", "Z_NEG", "DIR_NONE"]
    t = oracle.reactive_area_tensor(m)
    for d in range(6):
        assert float(rows[d]["rad"]) == pytest.approx(t[d], rel=1e-5)
    assert float(rows[6]["rad"]) == pytest.approx(oracle.reactive_area(m), rel=1e-5)
    assert float(rows[0]["porosity"]) == pytest.approx(float((m == 0).mean()), rel=1e-5)
    # --basic: one row per direction, no dir column.
    out2 = str(tmp_path / "b.csv")
    r = subprocess.run([build.CLI, "alpha", p, "-d", "xy", "--basic", "-o", out2], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    rows = list(csv.DictReader(open(out2)))
    assert len(rows) == 2 and list(rows[0]) == ["ID", "dimx", "dimy", "dimz", "porosity", "radBasic", "radBasicTime"]
    assert float(rows[0]["radBasic"]) == pytest.approx(oracle.reactive_area(m), rel=1e-5)


@pytest.mark.gpu
def test_cli_alpha_segmentinfo(gpu, oracle, tmp_path):
    from fast_gb300 import build
    m = np.empty((22, 26, 30), np.uint8)
    assert gpu.fast_gen_spheres(m.ctypes.data_as(C.c_void_p), 30, 26, 22, 8, 2.0, 4.0, 0.62) == Status.OK
    p = str(tmp_path / "v.bin")
    volume_io.save_volume_binary(p, m)
    out, info = str(tmp_path / "a.csv"), str(tmp_path / "seg.csv")
    r = subprocess.run([build.CLI, "alpha", p, "-d", "xy", "-o", out, "--segmentinfo", info], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rows = list(csv.DictReader(open(out)))
    assert list(rows[0])[-1] == "segmentVolumeRatio"
    labels, k = oracle.ccl_label(m, 255)
    table = oracle.ccl_boundary(labels, k)
    counts = np.bincount(labels.ravel(), minlength=k)
    n = m.size
    for row, d in zip(rows, [X_POS, Y_POS, 6]):
        want = counts[1:][table[d][1:] == 0].sum() / n
        assert float(row["segmentVolumeRatio"]) == pytest.approx(want, rel=1e-5, abs=1e-7)
    seg = list(csv.DictReader(open(info)))
    assert list(seg[0]) == ["ID", "atBoundary", "labelID", "maxX", "maxY", "maxZ", "minX", "minY", "minZ",
                            "voxelNum"]
    want_ids = [l for l in range(1, k) if table[6][l] == 0]
    assert [int(s["labelID"]) for s in seg] == want_ids
    for s in seg[:20]:
        l = int(s["labelID"])
        z, y, x = np.nonzero(labels == l)
        assert int(s["voxelNum"]) == len(x)
        assert (int(s["minX"]), int(s["minY"]), int(s["minZ"])) == (x.min(), y.min(), z.min())
        assert (int(s["maxX"]), int(s["maxY"]), int(s["maxZ"])) == (x.max() + 1, y.max() + 1, z.max() + 1)
        at = x.min() == 0 or y.min() == 0 or z.min() == 0 or x.max() == 29 or y.max() == 25 or z.max() == 21
        assert int(s["atBoundary"]) == int(at)


@pytest.mark.gpu
def test_cli_alpha_mesh(gpu, oracle, tmp_path):
    from collections import Counter
    from fast_gb300 import build
    m = np.empty((14, 16, 18), np.uint8)
    assert gpu.fast_gen_spheres(m.ctypes.data_as(C.c_void_p), 18, 16, 14, 4, 2.0, 3.5, 0.45) == Status.OK
    p = str(tmp_path / "v.bin")
    volume_io.save_volume_binary(p, m)
    obj = str(tmp_path / "s.obj")
    r = subprocess.run([build.CLI, "alpha", p, "--basic", "-o", str(tmp_path / "a.csv"), "--mesh", obj],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "Saving" in r.stdout and "Done." in r.stdout
    v, vn, f = [], [], []
    for line in open(obj):
        tag, *vals = line.split()
        if tag == "v":
            v.append([float(x) for x in vals])
        elif tag == "vn":
            vn.append([float(x) for x in vals])
        elif tag == "f":
            f.append([int(x) - 1 for x in vals])
    v, vn, f = np.array(v), np.array(vn), np.array(f)
    assert len(v) == len(vn) and len(f) > 0 and f.min() >= 0 and f.max() < len(v)
    # unit normals, or zero where a vertex only belongs to zero-area
    # triangles (cut points that coincide when a corner equals the isovalue)
    nrm = np.linalg.norm(vn, axis=1)
    assert np.all((np.abs(nrm - 1.0) < 1e-4) | (nrm == 0.0))
    # mesh frame: voxel size 1/max(padded dims) on every axis, centred
    pad = np.zeros((16, 18, 20), np.uint8)
    pad[1:-1, 1:-1, 1:-1] = m
    assert np.abs(v).max() <= 0.5 + 1e-6
    # the area of the OBJ triangles is the oracle's area of the padded field,
    # rescaled from per-axis units (1/n_a) to the mesh frame (1/max n)
    a = v[f[:, 1]] - v[f[:, 0]]
    b = v[f[:, 2]] - v[f[:, 0]]
    area_obj = 0.5 * np.linalg.norm(np.cross(a, b), axis=1).sum()
    nz, ny, nx = pad.shape
    d = 1.0 / max(pad.shape)
    scale = np.array([nx * d, ny * d, nz * d])          # mesh frame = per-axis frame * scale
    # per-triangle rescaling is anisotropic: compare through the oracle's own
    # triangle areas only when the volume is cubic; here check against a
    # direct recomputation in the per-axis frame instead
    area_axis = 0.5 * np.linalg.norm(np.cross(a / scale, b / scale), axis=1).sum()
    assert area_axis == pytest.approx(oracle.reactive_area(pad), rel=2e-4)
    assert area_obj > 0
    # closed surface: the boundary of the triangle set is empty, i.e. every
    # edge (by rounded position) of a nonzero-area triangle occurs an even
    # number of times (two, or more where surface sheets touch along an edge)
    key = np.round(v / d * 4096).astype(np.int64)
    nonzero = np.linalg.norm(np.cross(a, b), axis=1) > 1e-12
    edges = Counter()
    for t in f[nonzero]:
        pts = [tuple(key[i]) for i in t]
        for e in range(3):
            u, w = pts[e], pts[(e + 1) % 3]
            if u != w:
                edges[(min(u, w), max(u, w))] += 1
    assert edges and all(c % 2 == 0 for c in edges.values())
    assert sum(c == 2 for c in edges.values()) > 0.95 * len(edges)
