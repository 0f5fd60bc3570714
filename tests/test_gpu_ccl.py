"""GPU connected-component labelling (the reachability pre-pass) against the
CPU oracle's restatement of VolumeCCL_Label / VolumeCCL_BoundaryLabels:
labels, label count and the 7-row boundary table must be bit-identical."""
import numpy as np
import pytest

from fast_gb300 import ccl, volumes

pytestmark = pytest.mark.gpu


def _random(shape, p, seed, fg=0, bg=255):
    r = np.random.default_rng(seed).random(shape)
    return np.where(r < p, np.uint8(fg), np.uint8(bg))


CASES = [
    ("random_sparse", lambda: _random((23, 37, 41), 0.25, 1)),
    ("random_critical", lambda: _random((40, 33, 65), 0.31, 2)),   # near 3-D site percolation
    ("random_dense", lambda: _random((31, 29, 70), 0.7, 3)),
    ("spheres", lambda: volumes.spheres((48, 40, 56), seed=5, r_min=4.0, solid_fraction=0.65)),
    ("long_rows", lambda: _random((5, 7, 300), 0.5, 4)),              # runs crossing several 32-voxel chunks
    ("all_fg", lambda: np.zeros((9, 10, 11), np.uint8)),
    ("all_bg", lambda: np.full((9, 10, 11), 255, np.uint8)),
    ("single_fg", lambda: np.zeros((1, 1, 1), np.uint8)),
    ("single_bg", lambda: np.full((1, 1, 1), 255, np.uint8)),
    ("line_x", lambda: _random((1, 1, 97), 0.6, 6)),
    ("line_z", lambda: _random((97, 1, 1), 0.6, 7)),
    ("plane_xy", lambda: _random((1, 45, 45), 0.55, 8)),
    ("checker", lambda: ((np.indices((8, 9, 10)).sum(0) % 2) * 255).astype(np.uint8)),  # K = N/2 singletons
]


@pytest.mark.parametrize("name,make", CASES, ids=[c[0] for c in CASES])
def test_labels_bit_exact(gpu, oracle, name, make):
    m = make()
    got = ccl.get_volume_ccl(m, background=255)
    ref_labels, ref_n = oracle.ccl_label(m, background=255)
    assert got.num_labels == ref_n
    np.testing.assert_array_equal(got.labels, ref_labels)
    ref_bnd = oracle.ccl_boundary(ref_labels, ref_n)
    np.testing.assert_array_equal(got.boundary_label_mask, ref_bnd)


def test_background_zero(gpu, oracle):
    # components of the solid phase: background 0 (the reference's toggle
    # semantics with background = 0)
    m = _random((20, 26, 35), 0.45, 9)
    got = ccl.get_volume_ccl(m, background=0)
    ref_labels, ref_n = oracle.ccl_label(m, background=0)
    assert got.num_labels == ref_n
    np.testing.assert_array_equal(got.labels, ref_labels)


def test_dir_masks_and_boundary_volume(gpu, oracle):
    m = volumes.spheres((30, 34, 38), seed=12, r_min=3.0, solid_fraction=0.6)
    c = ccl.get_volume_ccl(m)
    ref_labels, ref_n = oracle.ccl_label(m)
    bnd = oracle.ccl_boundary(ref_labels, ref_n)
    from fast_gb300 import Dir
    both = c.get_dir_mask(Dir.X_NEG, Dir.X_POS)
    np.testing.assert_array_equal(both, bnd[1] & bnd[0])
    vol = ccl.generate_boundary_connected_volume(c, Dir.X_NEG)
    np.testing.assert_array_equal(vol, np.where(bnd[1][ref_labels] > 0, 255, 0).astype(np.uint8))
    inv = ccl.generate_boundary_connected_volume(c, Dir.X_NEG, invert_mask=True)
    sel = bnd[1].astype(bool)
    sel[1:] = ~sel[1:]
    np.testing.assert_array_equal(inv, np.where(sel[ref_labels], 255, 0).astype(np.uint8))


def test_device_entry_matches_host(gpu):
    torch = pytest.importorskip("torch")
    m = _random((37, 41, 43), 0.33, 13)
    host = ccl.get_volume_ccl(m)
    d_mask = torch.from_numpy(m).cuda()
    d_labels = torch.empty(m.shape, dtype=torch.int32, device="cuda")
    for _ in range(2):  # two calls in a row reuse nothing
        dev = ccl.get_volume_ccl_device(d_mask.data_ptr(), m.shape, d_labels.data_ptr())
        assert dev.num_labels == host.num_labels
        np.testing.assert_array_equal(d_labels.cpu().numpy().view(np.uint32), host.labels)
        np.testing.assert_array_equal(dev.boundary_label_mask, host.boundary_label_mask)


def test_many_components_boundary_retry(gpu, oracle):
    # more components than the first boundary buffer guess forces the retry
    m = ((np.indices((64, 128, 260)).sum(0) % 2) * 255).astype(np.uint8)
    c = ccl.get_volume_ccl(m)
    assert c.num_labels == (m == 0).sum() + 1 > (1 << 20)
    ref_labels, ref_n = oracle.ccl_label(m)
    np.testing.assert_array_equal(c.labels, ref_labels)


@pytest.mark.parametrize("shape,frac", [((96, 80, 150), 0.35), ((64, 64, 64), 0.2)])
def test_dominant_component_repeatable(gpu, oracle, shape, frac):
    """One component spanning most of the pore space: every join and run
    start walks to the same root, which is where the concurrent union-find
    races.  Several calls must give the same labels, equal to the oracle's."""
    m = volumes.spheres(shape, seed=21, r_min=3.0, r_max=6.0, solid_fraction=frac)
    ref_labels, ref_n = oracle.ccl_label(m)
    sizes = np.bincount(ref_labels.ravel())[1:]
    assert sizes.max() > 0.9 * sizes.sum()  # the case is the dominant-component one
    for _ in range(4):
        got = ccl.get_volume_ccl(m)
        assert got.num_labels == ref_n
        np.testing.assert_array_equal(got.labels, ref_labels)
