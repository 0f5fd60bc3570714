"""Batched solves of uneven volumes (fast_tau_solve_batch): every right-hand
side of the batch gives what it gives alone (bit-identical at a fixed slab
depth: its reductions never mix with another's), and matches the oracle
within the single-solve bounds."""
import numpy as np
import pytest

import fast_gb300 as ft
from fast_gb300 import volumes

pytestmark = pytest.mark.gpu


def _batch(seed, n=7):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        shape = tuple(int(v) for v in rng.integers(9, 40, size=3))
        m = volumes.spheres(shape, seed=int(rng.integers(1 << 30)), r_min=2.0, r_max=4.0,
                            solid_fraction=float(rng.uniform(0.35, 0.6)))
        out.append((m, ft.Dir(int(rng.integers(6)))))
    return out


@pytest.mark.parametrize("solver", [ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB])
@pytest.mark.parametrize("prec", [ft.Precision.F64, ft.Precision.MIXED])
def test_batch_equals_single(gpu, solver, prec):
    # A batch picks its slab depth for the whole launch, a volume solved alone
    # for itself, so the two differ only in the order of the dot-product
    # partial sums: equal within the rounding of a tol-1e-8 solve.
    vols = _batch(100 + int(prec) * 2 + int(solver))
    p = ft.TortuosityParams(tolerance=1e-8, precision=prec)
    batch = ft.solve_batch(vols, p, solver)
    assert len(batch) == len(vols)
    for (m, d), r in zip(vols, batch):
        single = ft.solve_directions(m, [d], p, solver)[0]
        assert r.status == single.status == ft.Status.OK
        assert r.porosity == single.porosity
        assert abs(r.tau - single.tau) <= 1e-6 * single.tau


def test_batch_is_bit_identical_at_fixed_depth(gpu, monkeypatch):
    # With the slab depth fixed, the right-hand sides of a batch never mix:
    # every result is bit-identical to the volume solved alone.
    monkeypatch.setenv("FAST_TAU_ZC", "8")
    vols = _batch(77, n=5)
    for solver in (ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB):
        p = ft.TortuosityParams(tolerance=1e-8, precision=ft.Precision.MIXED)
        batch = ft.solve_batch(vols, p, solver)
        for (m, d), r in zip(vols, batch):
            single = ft.solve_directions(m, [d], p, solver)[0]
            assert (r.tau, r.iterations, r.outer_steps) == (single.tau, single.iterations, single.outer_steps)


def test_batch_matches_oracle(gpu, oracle):
    vols = _batch(7, n=5)
    p = ft.TortuosityParams(tolerance=1e-10, precision=ft.Precision.F64)
    res = ft.solve_batch(vols, p, ft.DSOLVER_CG)
    for (m, d), r in zip(vols, res):
        ref = oracle.get_tortuosity(m, dir=int(d), solver=1, tol=1e-10)
        assert r.status == ft.Status.OK
        assert abs(r.tau - ref["tau"]) <= 1e-9 * abs(ref["tau"])
        assert abs(r.iterations - ref["iters"]) <= 2


def test_batch_mixed_accuracy(gpu, oracle):
    vols = _batch(8, n=6)
    p = ft.TortuosityParams(tolerance=1e-7, precision=ft.Precision.MIXED)
    for solver in (ft.DSOLVER_CG, ft.DSOLVER_BICGSTAB):
        res = ft.solve_batch(vols, p, solver)
        for (m, d), r in zip(vols, res):
            ref = oracle.get_tortuosity(m, dir=int(d), solver=1, tol=1e-10)
            assert r.status == ft.Status.OK
            assert abs(r.tau - ref["tau"]) <= 1e-5 * abs(ref["tau"])


def test_batch_device_entry(gpu):
    torch = pytest.importorskip("torch")
    vols = _batch(9, n=4)
    p = ft.TortuosityParams(tolerance=1e-8, precision=ft.Precision.MIXED)
    host = ft.solve_batch(vols, p, ft.DSOLVER_CG)
    dev_masks = [torch.from_numpy(m).cuda() for m, _ in vols]
    dev = ft.solve_batch_device([(t.data_ptr(), m.shape, d) for t, (m, d) in zip(dev_masks, vols)], p, ft.DSOLVER_CG)
    assert [(r.tau, r.iterations) for r in dev] == [(r.tau, r.iterations) for r in host]


def test_batch_failure_is_per_volume(gpu):
    # one volume that cannot converge in 3 iterations next to easy ones:
    # its status is reported, the others still succeed
    vols = _batch(10, n=3)
    hard = volumes.spheres((40, 40, 40), seed=3, r_min=2.0, r_max=3.0, solid_fraction=0.6)
    p = ft.TortuosityParams(tolerance=1e-12, max_iter=3, precision=ft.Precision.F64)
    res = ft.solve_batch([(hard, ft.Dir.X_POS)], p, ft.DSOLVER_CG)
    assert res[0].status == ft.Status.NO_CONVERGENCE and res[0].tau == 0.0
    p2 = ft.TortuosityParams(tolerance=1e-6, max_iter=10000, precision=ft.Precision.F64)
    res2 = ft.solve_batch(vols + [(np.zeros((5, 6, 7), np.uint8), ft.Dir.Y_NEG)], p2, ft.DSOLVER_CG)
    assert all(r.status == ft.Status.OK for r in res2)
    assert abs(res2[-1].tau - 1.0) < 1e-6   # all-pore volume: tau = 1
