"""ctypes binding of libstencilcuda.so (the C ABI declared in include/stencil_cuda.h).

The library is the only compute path: if it is missing or no sm_100-family GPU is present,
calls raise instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import _abi as A

import os

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libstencilcuda.so"
# the debug build (device-side bounds tests, STC_ERR_BOUNDS), loaded instead when STC_DEBUG_BOUNDS=1
LIB_DEBUG_PATH = Path(__file__).resolve().parent / "_build" / "debug" / "libstencilcuda_debug.so"
_lib = None


class StencilError(RuntimeError):
    """A nonzero status from the library."""

    def __init__(self, status: int, what: str = ""):
        self.status = status
        name = A.STATUS_NAMES.get(status, str(status))
        msg = f"{what}: {name}"
        if _lib is not None:
            msg += f" ({_lib.stc_strerror(status).decode()})"
            if status == -6:
                msg += f" [cudaError {_lib.stc_last_cuda_error()}]"
        super().__init__(msg)


class ArgumentError(StencilError, A.ArgumentError):
    """The statuses that mirror the reference's ArgumentErrors (sizes, radius, kernel length)."""


def load(path: str | Path | None = None):
    """Load the shared library (built by `stencils_gb300.build.build()`)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else (LIB_DEBUG_PATH if os.environ.get("STC_DEBUG_BOUNDS") == "1" else LIB_PATH)
    if not p.exists():
        raise RuntimeError(f"libstencilcuda.so not built ({p}); run __graft_entry__.build()")
    lib = C.CDLL(str(p))
    P = C.POINTER
    vp = C.c_void_p
    sig = {
        "stc_abi_version": ([], C.c_int),
        "stc_strerror": ([C.c_int], C.c_char_p),
        "stc_last_cuda_error": ([], C.c_int),
        "stc_debug_bounds": ([], C.c_int),
        "stc_debug_report_bounds": ([vp], C.c_int),
        "stc_release_workspace": ([], C.c_int),
        "stc_result_dtype": ([C.c_int32, C.c_int32, C.c_int32], C.c_int),
        "stc_neighbor_dtype": ([C.c_int32, P(A.BcDesc)], C.c_int),
        "stc_map": ([P(A.Grid), P(A.Grid), C.c_int32, P(A.StencilDesc), P(A.OpDesc), P(A.BcDesc), vp, C.c_uint32],
                    C.c_int),
        "stc_map_steps": ([P(A.Grid), P(A.Grid), P(A.StencilDesc), P(A.OpDesc), P(A.BcDesc), C.c_int64,
                           P(C.c_int32), vp, C.c_uint32], C.c_int),
        "stc_update_boundary": ([P(A.Grid), C.c_int32, P(A.BcDesc), vp, C.c_uint32], C.c_int),
        "stc_grid_upload": ([P(A.Grid), vp, vp, C.c_uint32], C.c_int),
        "stc_grid_download": ([vp, P(A.Grid), vp, C.c_uint32], C.c_int),
        "stc_map_terms": ([P(A.TermDesc), C.c_int32, P(A.Grid), C.c_int32, vp, C.c_uint32], C.c_int),
        "stc_scatter": ([P(A.Grid), P(A.Grid), P(A.StencilDesc), vp, P(A.BcDesc), vp, C.c_uint32], C.c_int),
        "stc_mass": ([P(A.Grid), C.c_int32, P(A.BcDesc), P(C.c_double), vp], C.c_int),
        "stc_life_steps_noalloc": ([P(A.Grid), P(A.Grid), P(A.StencilDesc), P(A.OpDesc), P(A.BcDesc), C.c_int64,
                                    P(C.c_int32), vp], C.c_int),
        "stc_profile_enable": ([C.c_int32], C.c_int),
        "stc_profile_report": ([C.c_char_p, C.c_size_t], C.c_int),
        "stc_batch_create": ([P(vp)], C.c_int),
        "stc_batch_destroy": ([vp], C.c_int),
        "stc_batch_add": ([vp, P(A.Grid), P(A.Grid), P(A.StencilDesc), P(A.OpDesc), P(A.BcDesc), C.c_int64],
                          C.c_int),
        "stc_batch_plan": ([vp, C.c_int32, vp], C.c_int),
        "stc_batch_run": ([vp, vp, C.c_uint32], C.c_int),
        "stc_batch_result": ([vp, C.c_int32, P(C.c_int32)], C.c_int),
        "stc_batch_run_sequential": ([vp, vp], C.c_int),
        "stc_server_create": ([P(vp), C.c_double, C.c_int32], C.c_int),
        "stc_server_destroy": ([vp], C.c_int),
        "stc_server_submit": ([vp, P(A.JobDesc), P(C.c_int64)], C.c_int),
        "stc_server_poll": ([vp, C.c_int64], C.c_int),
        "stc_server_fetch": ([vp, C.c_int64, vp, C.c_size_t, P(C.c_double)], C.c_int),
        "stc_server_fetch_buffer": ([vp, C.c_int64, P(vp), P(C.c_size_t), P(C.c_double)], C.c_int),
        "stc_server_release_buffer": ([vp], C.c_int),
        "stc_server_ready": ([vp, P(C.c_int64), C.c_int32, C.c_double, P(C.c_int32)], C.c_int),
        "stc_server_cancel": ([vp, C.c_int64], C.c_int),
        "stc_server_drain": ([vp, C.c_double], C.c_int),
        "stc_server_stats": ([vp, P(C.c_int64), P(C.c_int64), P(C.c_int64), P(C.c_int64)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def check(status: int, what: str):
    if status != 0:
        if status in (-1, -2, -3):
            raise ArgumentError(status, what)
        if status == -4:
            err = StencilError(status, what)
            raise NotImplementedError(str(err))
        raise StencilError(status, what)
    return status


def profile_enable(on: bool = True):
    load().stc_profile_enable(1 if on else 0)


def profile_report() -> dict:
    """Per-kernel {launches, ms, alg_bytes, updates} recorded since profile_enable(True)."""
    import json
    lib = load()
    n = lib.stc_profile_report(None, 0)
    if n < 0:
        check(n, "profile_report")
    buf = C.create_string_buffer(max(n, 2) + 16)
    check(lib.stc_profile_report(buf, len(buf)), "profile_report")
    return json.loads(buf.value.decode())


def current_stream_handle():
    """torch's current CUDA stream as a raw cudaStream_t."""
    import torch
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)
