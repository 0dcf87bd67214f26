"""Batched runs: many independent SwitchingStencilArray loops as one persistent, graph-captured launch.

No counterpart in the reference, where each job is its own `A = mapstencil!(f, A)` loop.  Every job's
result is bit-identical to running it alone with `mapstencil_(f, S, steps=n)`.
"""
from __future__ import annotations

import ctypes as C

from . import _abi as A
from . import _lib
from .array import SwitchingStencilArray
from .boundary import Conditional
from .ops import as_reduction


class Batch:
    def __init__(self):
        self._lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self._lib.stc_batch_create(C.byref(h)), "stc_batch_create")
        self._h = h
        self._jobs = []        # (S, lowered stencil, op, bc, grids) kept alive

    def add(self, f, S: SwitchingStencilArray, steps: int) -> int:
        """Queue `steps` iterations of S = mapstencil_(f, S); returns the job index."""
        red = as_reduction(f)
        if not isinstance(S.padding, Conditional):
            raise NotImplementedError("batched jobs use Conditional padding")
        st = A.LoweredStencil(S.stencil)
        op = A.lower_op(red)
        bc = A.lower_bc(S.boundary, S.padding, A.torch_dtype_code(S.source.dtype))
        ga, gb = A.grid_from_torch(S.source), A.grid_from_torch(S.dest)
        rc = self._lib.stc_batch_add(self._h, C.byref(ga), C.byref(gb), C.byref(st.desc), C.byref(op),
                                     C.byref(bc), int(steps))
        if rc < 0:
            _lib.check(rc, "stc_batch_add")
        self._jobs.append((S, st, op, bc, ga, gb))
        return rc

    def plan(self, autotune: bool = True):
        _lib.check(self._lib.stc_batch_plan(self._h, 1 if autotune else 0, _lib.current_stream_handle()),
                   "stc_batch_plan")

    def run(self, sync: bool = True):
        _lib.check(self._lib.stc_batch_run(self._h, _lib.current_stream_handle(), 0 if sync else A.STC_ASYNC),
                   "stc_batch_run")

    def run_sequential(self):
        """The plain path: each job as its own synchronising mapstencil_ loop."""
        _lib.check(self._lib.stc_batch_run_sequential(self._h, _lib.current_stream_handle()),
                   "stc_batch_run_sequential")

    def result(self, idx: int) -> SwitchingStencilArray:
        """The job's array after the batch ran (switched if its result is in the second parent)."""
        out = C.c_int32(0)
        _lib.check(self._lib.stc_batch_result(self._h, idx, C.byref(out)), "stc_batch_result")
        S = self._jobs[idx][0]
        return S.switch() if out.value else S

    def __len__(self):
        return len(self._jobs)

    def close(self):
        if self._h:
            self._lib.stc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # pragma: no cover
            pass
