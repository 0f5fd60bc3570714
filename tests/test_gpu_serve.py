"""Serving context (continuous batching): requests that arrive while others
are on the GPU are admitted as slots and memory free up, share the launches,
and each result is the same as solving that request alone."""
import numpy as np
import pytest

import fast_gb300 as ft
from fast_gb300 import volumes
from fast_gb300.serve import TauServer

pytestmark = pytest.mark.gpu


def _requests(seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        edge = np.exp(rng.uniform(np.log(12), np.log(44), size=3)).astype(int)
        shape = tuple(int(v) for v in edge)
        if rng.random() < 0.5:
            m = volumes.spheres(shape, seed=int(rng.integers(1 << 30)), r_min=2.0, r_max=4.0,
                                solid_fraction=float(rng.uniform(0.4, 0.6)))
        else:
            m = volumes.ellipsoids(shape, int(rng.integers(1 << 30)), 4.0, float(rng.uniform(0.3, 1.0)),
                                   float(rng.uniform(0.4, 0.6)))
        solver = ft.DSOLVER_CG if rng.random() < 0.5 else ft.DSOLVER_BICGSTAB
        out.append((m, ft.Dir(int(rng.integers(6))), solver))
    return out


def _alone(m, d, solver, prec, tol):
    p = ft.TortuosityParams(tolerance=tol, precision=prec)
    return ft.solve_directions(m, [d], p, solver)[0]


@pytest.mark.parametrize("prec", [ft.Precision.MIXED, ft.Precision.F64])
def test_results_equal_alone(gpu, prec):
    reqs = _requests(1 + int(prec), 10)
    with TauServer(precision=prec, tolerance=1e-7, chunk=8) as srv:
        tickets = {srv.submit(m, d, s): k for k, (m, d, s) in enumerate(reqs)}
        done = srv.drain()
    assert sorted(c.ticket for c in done) == sorted(tickets)
    for c in done:
        m, d, s = reqs[tickets[c.ticket]]
        ref = _alone(m, d, s, prec, 1e-7)
        assert c.result.status == ref.status == ft.Status.OK
        assert (c.result.tau, c.result.iterations, c.result.porosity) == (ref.tau, ref.iterations, ref.porosity)


def test_arrivals_while_busy_overlap(gpu):
    reqs = _requests(5, 12)
    with TauServer(tolerance=1e-7, chunk=4) as srv:
        tickets = {}
        done = []
        max_inflight = 0
        for k, (m, d, s) in enumerate(reqs):
            tickets[srv.submit(m, d, s)] = k
            done.extend(srv.poll())   # a step between arrivals
            max_inflight = max(max_inflight, srv.stats()["inflight"])
        done.extend(srv.drain())
    assert max_inflight > 1   # later arrivals joined solves already on the GPU
    admits = sorted(c.t_admit for c in done)
    finishes = sorted(c.t_done for c in done)
    assert admits[-1] > finishes[0] or max_inflight > 1
    for c in done:
        m, d, s = reqs[tickets[c.ticket]]
        ref = _alone(m, d, s, ft.Precision.MIXED, 1e-7)
        assert (c.result.tau, c.result.iterations) == (ref.tau, ref.iterations)


def test_hbm_budget_admission(gpu):
    reqs = _requests(9, 5)
    with TauServer(tolerance=1e-6, hbm_budget=1) as srv:   # nothing fits: one at a time
        for m, d, s in reqs:
            srv.submit(m, d, s)
        seen = 0
        done = []
        while srv.busy():
            done.extend(srv.poll())
            seen = max(seen, srv.stats()["inflight"])
    assert seen == 1
    assert all(c.result.status == ft.Status.OK for c in done)
    # admitted strictly one after another
    ordered = sorted(done, key=lambda c: c.t_admit)
    for a, b in zip(ordered, ordered[1:]):
        assert b.t_admit >= a.t_done


def test_failure_is_per_request(gpu):
    reqs = _requests(11, 3)
    hard = volumes.spheres((36, 36, 36), seed=4, r_min=2.0, r_max=3.0, solid_fraction=0.6)
    with TauServer(tolerance=1e-12, max_iter=5, precision=ft.Precision.F64) as srv:
        t_hard = srv.submit(hard, ft.Dir.X_POS, ft.DSOLVER_CG)
        done = srv.drain()
    assert done[0].ticket == t_hard and done[0].result.status == ft.Status.NO_CONVERGENCE
    with TauServer(tolerance=1e-6) as srv:
        for m, d, s in reqs:
            srv.submit(m, d, s)
        assert all(c.result.status == ft.Status.OK for c in srv.drain())
