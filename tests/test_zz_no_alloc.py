"""The allocation-free pore count, for callers that cannot allocate device
memory (an application whose own allocator has reserved all of the GPU's
memory, or a plug-in host that forbids device allocation): called through the
C ABI on a device mask, it must give the same
count as the allocating fast_porosity, on two calls in a row that share its
static scratch.  Counts are integers, so the comparison is exact.

This file sorts last so that a run stopping at the first failure has already
run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _allocating_count(L, m):
    nz, ny, nx = m.shape
    cnt = C.c_uint64(0)
    phi = C.c_double(0)
    assert L.fast_porosity(m.ctypes.data_as(C.c_void_p), nx, ny, nz, C.byref(phi), C.byref(cnt)) == 0
    return cnt.value, phi.value


def test_noalloc_pore_count_matches_fast_porosity(gpu):
    torch = pytest.importorskip("torch")
    from fast_gb300 import volumes
    L = gpu
    vols = [
        volumes.spheres((40, 48, 70), seed=31, r_min=3.0, solid_fraction=0.55),     # two blocks and a tail
        ((np.random.default_rng(32).random((33, 17, 129)) < 0.3) * 255).astype(np.uint8),
    ]
    for m in vols:  # two calls in a row on the shared scratch
        nz, ny, nx = m.shape
        d = torch.from_numpy(m).cuda()
        torch.cuda.synchronize()
        cnt = C.c_uint64(0)
        phi = C.c_double(0)
        st = L.fast_porosity_device_noalloc(C.c_void_p(d.data_ptr()), nx, ny, nz, C.byref(cnt), C.byref(phi), None)
        assert st == 0, L.fast_last_error()
        ref_cnt, ref_phi = _allocating_count(L, m)
        assert cnt.value == ref_cnt == int((m == 0).sum())
        assert phi.value == ref_phi


def test_noalloc_on_a_side_stream_with_many_blocks(gpu):
    """About 100 M voxels (1526 blocks of the last-block-done reduction) on a
    non-default stream, twice in a row, against the allocating count."""
    torch = pytest.importorskip("torch")
    L = gpu
    rng = np.random.default_rng(33)
    m = ((rng.random((400, 500, 500), dtype=np.float32) < 0.37) * 255).astype(np.uint8)
    nz, ny, nx = m.shape
    ref_cnt, ref_phi = _allocating_count(L, m)
    assert ref_cnt == int((m == 0).sum())
    side = torch.cuda.Stream()
    d = torch.from_numpy(m).cuda()
    side.wait_stream(torch.cuda.current_stream())
    for _ in range(2):
        cnt = C.c_uint64(0)
        phi = C.c_double(0)
        st = L.fast_porosity_device_noalloc(C.c_void_p(d.data_ptr()), nx, ny, nz, C.byref(cnt), C.byref(phi),
                                            C.c_void_p(side.cuda_stream))
        assert st == 0, L.fast_last_error()
        assert cnt.value == ref_cnt
        assert phi.value == ref_phi


def test_noalloc_rejects_volumes_beyond_its_scratch(gpu):
    torch = pytest.importorskip("torch")
    L = gpu
    d = torch.zeros(16, dtype=torch.uint8, device="cuda")
    cnt = C.c_uint64(7)
    # 2048 x 1024 x 1024 voxels: above the static scratch's limit; rejected
    # before any GPU work touches the (small) buffer.
    st = L.fast_porosity_device_noalloc(C.c_void_p(d.data_ptr()), 2048, 1024, 1024, C.byref(cnt), None, None)
    assert st == 8
    assert b"no-allocation limit" in L.fast_last_error()
    assert cnt.value == 7
