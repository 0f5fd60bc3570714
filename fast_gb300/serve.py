"""Serving: continuous batching of tortuosity requests on one GPU
(fast_ctx_* of libfasttau.so).

    srv = TauServer(tolerance=1e-6)
    t = srv.submit(mask, Dir.X_POS, DSOLVER_CG)
    while srv.busy():
        for done in srv.poll():
            print(done.ticket, done.result.tau, done.latency)

Each poll is one scheduling step: finished solves are retired and returned,
queued requests are admitted while their device footprint fits the HBM
budget, and every in-flight solve advances by `chunk` iterations in shared
launches.  A request's result is identical to solving it alone."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import _native
from .tau import DSOLVER_BICGSTAB, DiffusionSolverType, Dir, Precision, Status, TauResult, _as_mask


@dataclass
class Completion:
    ticket: int
    result: TauResult
    solver: DiffusionSolverType
    t_submit: float
    t_admit: float
    t_done: float

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


class TauServer:
    def __init__(self, precision: Precision = Precision.MIXED, tolerance: float = 1e-6, max_iter: int = 10000,
                 chunk: int = 16, max_inflight: int = 256, hbm_budget: int = 0, d0: float = None, d1: float = None):
        L = _native.lib()
        cfg = _native.fast_ctx_config()
        L.fast_ctx_config_init(C.byref(cfg))
        cfg.precision = int(precision)
        cfg.tolerance = tolerance
        cfg.max_iter = max_iter
        cfg.chunk = chunk
        cfg.max_inflight = max_inflight
        cfg.hbm_budget = hbm_budget
        if d0 is not None:
            cfg.d0 = d0
        if d1 is not None:
            cfg.d1 = d1
        h = C.c_void_p()
        st = L.fast_ctx_create(C.byref(cfg), C.byref(h))
        if st != 0:
            raise RuntimeError(f"fast_ctx_create: {_native.last_error()}")
        self._h = h
        self._cap = max(1, max_inflight)
        self._buf = (_native.fast_ctx_completion * self._cap)()
        self._outstanding = 0

    def submit(self, mask, dir: Dir, solver: DiffusionSolverType = DSOLVER_BICGSTAB) -> int:
        m = _as_mask(mask)
        if m is None:
            raise TypeError("mask must be a 3-D uint8 array [z, y, x]")
        nz, ny, nx = m.shape
        t = C.c_uint64(0)
        st = _native.lib().fast_ctx_submit(self._h, m.ctypes.data_as(C.c_void_p), nx, ny, nz, int(dir), int(solver),
                                           C.byref(t))
        if st != 0:
            raise RuntimeError(f"fast_ctx_submit: {_native.last_error()}")
        self._outstanding += 1
        return int(t.value)

    def poll(self) -> List[Completion]:
        n = C.c_int32(0)
        st = _native.lib().fast_ctx_poll(self._h, self._buf, self._cap, C.byref(n))
        if st != 0:
            raise RuntimeError(f"fast_ctx_poll: {_native.last_error()}")
        out = []
        for k in range(n.value):
            c = self._buf[k]
            r = c.result
            out.append(Completion(int(c.ticket), TauResult(r.tau, r.porosity, r.rel_residual, int(r.iterations),
                                                           int(r.outer_steps), Status(r.status), Dir(c.dir)),
                                  DiffusionSolverType(c.solver), c.t_submit, c.t_admit, c.t_done))
        self._outstanding -= len(out)
        return out

    def stats(self) -> dict:
        s = _native.fast_ctx_stats()
        _native.lib().fast_ctx_query(self._h, C.byref(s))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def now(self) -> float:
        return self.stats()["now"]

    def busy(self) -> bool:
        return self._outstanding > 0

    def drain(self) -> List[Completion]:
        out = []
        while self.busy():
            out.extend(self.poll())
        return out

    def close(self):
        if self._h:
            _native.lib().fast_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


__all__ = ["TauServer", "Completion"]
