"""TIFF-folder input (loadTiffFolder, VolumeIO.cpp:197-254) and binarize
(Volume.cpp:478-486, Volume.cu:157-183).

CPU part: libfasttau's TIFF reader (host code, no GPU call) decodes
hand-assembled files byte for byte, every layout the test writer makes, and
the folder rules (byte-wise name order, case-sensitive .tif/.tiff), and
refuses what it does not read.  GPU part: fast_binarize / fast_binarize_device
equal the oracle's rule on aligned and unaligned buffers, and `fast tau` on a
TIFF folder gives the rows of the same volume binarized and saved as .bin."""
import csv
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from fast_gb300 import Status, volume_io

from tiffs import tiff_bytes, write_folder

# A 3x2 little-endian slice assembled by hand: header (IFD at 8), six
# entries (width 3, height 2, 8 bits, no compression, one strip at 86 of 6
# bytes), no next IFD, then the pixels.
GOLDEN_II = bytes.fromhex(
    "49492a0008000000" "0600"
    "000103000100000003000000" "010103000100000002000000" "020103000100000008000000"
    "030103000100000001000000" "110104000100000056000000" "170104000100000006000000"
    "00000000" "1020304050ff")
# The same slice big-endian with one row per strip (RowsPerStrip 1): the two
# strip offsets (at 0x62) and byte counts (at 0x6a) follow the directory,
# then the rows at 0x72 and 0x75.
GOLDEN_MM = bytes.fromhex(
    "4d4d002a00000008" "0007"
    "010000030000000100030000" "010100030000000100020000" "010200030000000100080000"
    "010300030000000100010000" "011100040000000200000062" "011600030000000100010000"
    "01170004000000020000006a" "00000000"
    "0000007200000075" "0000000300000003" "1020304050ff")


def read_folder(native, folder):
    nx, ny, nz = C.c_int64(), C.c_int64(), C.c_int64()
    st = native.fast_tiff_folder_info(os.fsencode(str(folder)), C.byref(nx), C.byref(ny), C.byref(nz))
    if st != Status.OK:
        return st, None
    out = np.full((nz.value, ny.value, nx.value), 7, np.uint8)
    st = native.fast_tiff_folder_read(os.fsencode(str(folder)), out.ctypes.data_as(C.c_void_p), out.nbytes)
    return st, out


def test_golden_slices(native, tmp_path):
    expect = np.array([[0x10, 0x20, 0x30], [0x40, 0x50, 0xFF]], np.uint8)
    for k, raw in enumerate((GOLDEN_II, GOLDEN_MM)):
        d = tmp_path / f"g{k}"
        d.mkdir()
        (d / "s.tif").write_bytes(raw)
        st, v = read_folder(native, d)
        assert st == Status.OK, native.fast_last_error()
        assert v.shape == (1, 2, 3)
        np.testing.assert_array_equal(v[0], expect)


def test_writer_matches_golden():
    # The test writer's minimal form reproduces the hand-made file's pixels.
    img = np.array([[0x10, 0x20, 0x30], [0x40, 0x50, 0xFF]], np.uint8)
    raw = tiff_bytes(img, extra_fields=False)
    assert raw[:4] == GOLDEN_II[:4] and raw[8:14] == GOLDEN_II[86:92]


@pytest.mark.parametrize("kw", [
    dict(),
    dict(big_endian=True),
    dict(rows_per_strip=3),
    dict(rows_per_strip=1, long_fields=True),
    dict(big_endian=True, rows_per_strip=4, long_fields=True),
    dict(samples=3, planar=1),
    dict(samples=3, planar=2, rows_per_strip=5),
    dict(samples=2, planar=1, big_endian=True, rows_per_strip=2),
    dict(omit_counts=True),
])
def test_layouts(native, tmp_path, kw):
    kw = dict(kw)
    spp = kw.pop("samples", 1)
    rng = np.random.default_rng(len(str(kw)) + spp)
    vol = rng.integers(0, 256, size=(4, 13, 11) + ((spp,) if spp > 1 else ()), dtype=np.uint8)
    write_folder(tmp_path, vol, **kw)
    st, got = read_folder(native, tmp_path)
    assert st == Status.OK, native.fast_last_error()
    np.testing.assert_array_equal(got, vol[..., 0] if spp > 1 else vol)


def test_folder_rules(native, tmp_path):
    a = np.full((5, 6), 1, np.uint8)
    b = np.full((5, 6), 2, np.uint8)
    c = np.full((5, 6), 3, np.uint8)
    (tmp_path / "b.tif").write_bytes(tiff_bytes(b))
    (tmp_path / "a.tiff").write_bytes(tiff_bytes(a))
    (tmp_path / "B.tif").write_bytes(tiff_bytes(c))     # 'B' < 'a' byte-wise: first
    (tmp_path / "c.TIF").write_bytes(tiff_bytes(c))     # extension is case-sensitive: skipped
    (tmp_path / "notes.txt").write_text("x")
    (tmp_path / "dir.tif").mkdir()                      # a directory: skipped
    st, v = read_folder(native, tmp_path)
    assert st == Status.OK, native.fast_last_error()
    assert v.shape == (3, 5, 6)
    assert [int(s[0, 0]) for s in v] == [3, 1, 2]


def test_refusals(native, tmp_path):
    img = np.arange(48, dtype=np.uint8).reshape(6, 8)
    cases = {
        "bits16": (tiff_bytes(img.astype(np.uint16), bits=16), Status.BAD_TYPE),
        "lzw": (tiff_bytes(img, compression=5), Status.IO_ERROR),
        "tiled": (tiff_bytes(img, tiled=True), Status.IO_ERROR),
        "truncated": (tiff_bytes(img)[:20], Status.IO_ERROR),
        "notiff": (b"PK\x03\x04 not a tiff at all", Status.IO_ERROR),
    }
    for name, (raw, want) in cases.items():
        d = tmp_path / name
        d.mkdir()
        (d / "s.tif").write_bytes(raw)
        st, _ = read_folder(native, d)
        assert st == want, (name, native.fast_last_error())
        assert native.fast_last_error()
    # Slices of different sizes; an empty folder; a missing folder.
    d = tmp_path / "mixed"
    d.mkdir()
    (d / "a.tif").write_bytes(tiff_bytes(img))
    (d / "b.tif").write_bytes(tiff_bytes(img[:5]))
    assert read_folder(native, d)[0] == Status.IO_ERROR
    (tmp_path / "empty").mkdir()
    assert read_folder(native, tmp_path / "empty")[0] == Status.IO_ERROR
    assert read_folder(native, tmp_path / "absent")[0] == Status.IO_ERROR
    # Too small an output buffer.
    out = np.empty(10, np.uint8)
    st = native.fast_tiff_folder_read(os.fsencode(str(d)), out.ctypes.data_as(C.c_void_p), out.nbytes)
    assert st == Status.BAD_ARG


def test_oracle_binarize_rule(oracle):
    v = np.arange(256, dtype=np.uint8)
    np.testing.assert_array_equal(oracle.binarize(v, 1.0), np.where(v == 255, 255, 0))
    # uchar(0.5f * 255) = 127
    np.testing.assert_array_equal(oracle.binarize(v, 0.5), np.where(v >= 127, 255, 0))
    assert (oracle.binarize(v, 0.0) == 255).all()
    np.testing.assert_array_equal(oracle.binarize(v, 7.0), oracle.binarize(v, 1.0))


# ---------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("n", [0, 1, 15, 16, 17, 4096 + 5, 3_000_001])
@pytest.mark.parametrize("threshold", [1.0, 0.5, 0.0, 2.0])
def test_binarize_host(gpu, oracle, n, threshold):
    rng = np.random.default_rng(n)
    v = rng.integers(0, 256, size=n, dtype=np.uint8)
    v[:: 7] = 255
    want = oracle.binarize(v, threshold)
    got = v.copy()
    st = gpu.fast_binarize(got.ctypes.data_as(C.c_void_p), got.size, threshold)
    assert st == Status.OK, gpu.fast_last_error()
    np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("offset", [0, 1, 3, 15])
def test_binarize_device_unaligned(gpu, oracle, offset):
    import torch
    rng = np.random.default_rng(offset)
    n = 1 << 20
    host = rng.integers(0, 256, size=n + 64, dtype=np.uint8)
    d = torch.from_numpy(host.copy()).cuda()
    view = d[offset:offset + n + 7]
    s = torch.cuda.current_stream()
    st = gpu.fast_binarize_device(C.c_void_p(view.data_ptr()), view.numel(), 1.0, C.c_void_p(s.cuda_stream))
    assert st == Status.OK, gpu.fast_last_error()
    torch.cuda.synchronize()
    got = d.cpu().numpy()
    want = host.copy()
    want[offset:offset + n + 7] = oracle.binarize(host[offset:offset + n + 7])
    np.testing.assert_array_equal(got, want)


@pytest.mark.gpu
def test_load_tiff_folder_binarized_tau(gpu, oracle, tmp_path):
    import fast_gb300 as ft
    rng = np.random.default_rng(5)
    raw = rng.integers(0, 256, size=(20, 24, 28), dtype=np.uint8)
    raw[raw > 140] = 255                    # about 45 % solid after binarize
    write_folder(tmp_path, raw, big_endian=True, rows_per_strip=5)
    vol = volume_io.load_tiff_folder(str(tmp_path), binarize=True)
    np.testing.assert_array_equal(vol.data, oracle.binarize(raw))
    prm = ft.TortuosityParams(dir=ft.Dir.X_POS, tolerance=1e-10)
    tau = ft.get_tortuosity(vol, prm, ft.DSOLVER_CG)
    ref = oracle.get_tortuosity(vol.data, dir=0, tol=1e-10)
    assert ref["status"] == 0 and tau > 0
    assert abs(tau - ref["tau"]) <= 1e-9 * ref["tau"]


@pytest.mark.gpu
def test_cli_tiff_folder_equals_bin(gpu, oracle, tmp_path):
    from fast_gb300 import build
    rng = np.random.default_rng(9)
    raw = rng.integers(0, 256, size=(16, 18, 20), dtype=np.uint8)
    raw[raw > 120] = 255
    folder = tmp_path / "slices"
    write_folder(folder, raw, rows_per_strip=4)
    binp = str(tmp_path / "same.bin")
    volume_io.save_volume_binary(binp, oracle.binarize(raw))
    rows = {}
    for name, inp in (("tiff", str(folder)), ("bin", binp)):
        out = str(tmp_path / f"{name}.csv")
        r = subprocess.run([build.CLI, "tau", inp, "-d", "xyz", "-o", out], capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr
        with open(out) as f:
            rows[name] = list(csv.DictReader(f))
    assert len(rows["tiff"]) == 3
    for a, b in zip(rows["tiff"], rows["bin"]):
        assert a["ID"] == str(folder)
        for k in ("dimx", "dimy", "dimz", "dir", "porosity", "tau", "tauIter"):
            assert a[k] == b[k], k
        assert float(a["tau"]) > 0
