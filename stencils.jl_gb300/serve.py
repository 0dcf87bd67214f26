"""Serving: continuous batching of stencil jobs with device-resident state (stc_server_* in the C ABI).

No counterpart in the reference.  Jobs are host grids (numpy, Julia axis order); the server admits
them by an HBM budget, keeps their state on the GPU across batched ticks, and returns each result
with its latency from submission.  Each result equals running the job alone.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _abi as A
from . import _lib
from .boundary import Conditional
from .ops import as_reduction


class Server:
    def __init__(self, hbm_fraction: float = 0.8, steps_per_tick: int = 16):
        self._lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self._lib.stc_server_create(C.byref(h), float(hbm_fraction), int(steps_per_tick)),
                   "stc_server_create")
        self._h = h
        self._meta = {}

    def submit(self, grid: np.ndarray, stencil, f, boundary, steps: int, code: int | None = None) -> int:
        """Queue `steps` iterations of mapstencil_(f, ·) on a copy of `grid` (2D, Julia axis order).
        `code` overrides the element type (A.BF16 for bfloat16 bit patterns held as uint16)."""
        red = as_reduction(f)
        a = np.asarray(grid)
        # a column-major view (axis 0 contiguous, e.g. a corner of a larger Fortran array) is sent as is:
        # the server copies its rows straight from this memory; anything else is made column-major first
        if a.ndim != 2 or a.strides[0] != a.itemsize or a.strides[1] % a.itemsize or a.strides[1] < a.shape[0] * a.itemsize:
            a = np.asfortranarray(a)
        code = A.numpy_dtype_code(a.dtype) if code is None else code
        job = A.JobDesc()
        job.grid = A.grid_from_numpy(a, code)
        st = A.LoweredStencil(stencil)
        job.stencil = st.desc
        job.op = A.lower_op(red)
        job.bc = A.lower_bc(boundary, Conditional(), code)
        job.nsteps = int(steps)
        out = C.c_int64(0)
        _lib.check(self._lib.stc_server_submit(self._h, C.byref(job), C.byref(out)), "stc_server_submit")
        self._meta[out.value] = (a.shape, a.dtype, code)
        return out.value

    def poll(self, job_id: int) -> bool:
        rc = self._lib.stc_server_poll(self._h, job_id)
        if rc < 0:
            _lib.check(rc, "stc_server_poll")
        return rc == 1

    def ready(self, timeout_s: float = 0.0, max_ids: int = 4096) -> list:
        """Ids of jobs that finished, failed or were cancelled since the last call (a completion queue:
        each id once), waiting up to timeout_s for the first."""
        ids = (C.c_int64 * max_ids)()
        n = C.c_int32(0)
        _lib.check(self._lib.stc_server_ready(self._h, ids, max_ids, float(timeout_s), C.byref(n)), "stc_server_ready")
        return list(ids[:n.value])

    def fetch(self, job_id: int):
        """(result array, latency in seconds); raises StencilError(BUSY) if not finished.

        The array is a view of the pinned host buffer the server copied the result into (no further copy);
        the buffer returns to the library's pool when the array and its views are gone."""
        shape, dtype, code = self._meta[job_id]
        ptr, nbytes, lat = C.c_void_p(), C.c_size_t(0), C.c_double(0.0)
        _lib.check(self._lib.stc_server_fetch_buffer(self._h, job_id, C.byref(ptr), C.byref(nbytes), C.byref(lat)),
                   "stc_server_fetch")
        del self._meta[job_id]
        raw = (C.c_char * nbytes.value).from_address(ptr.value)
        weakref.finalize(raw, self._lib.stc_server_release_buffer, C.c_void_p(ptr.value))
        out = np.frombuffer(raw, dtype=dtype).reshape(shape, order="F")
        return out, lat.value

    def cancel(self, job_id: int):
        _lib.check(self._lib.stc_server_cancel(self._h, job_id), "stc_server_cancel")

    def drain(self, timeout_s: float = 60.0):
        _lib.check(self._lib.stc_server_drain(self._h, float(timeout_s)), "stc_server_drain")

    def stats(self) -> dict:
        v = [C.c_int64(0) for _ in range(4)]
        _lib.check(self._lib.stc_server_stats(self._h, *[C.byref(x) for x in v]), "stc_server_stats")
        return {"admitted": v[0].value, "finished": v[1].value, "ticks": v[2].value, "peak_bytes": v[3].value}

    def close(self):
        if self._h:
            self._lib.stc_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:  # pragma: no cover
            pass
