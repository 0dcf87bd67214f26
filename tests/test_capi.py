"""The C-ABI library: it loads without a GPU, exports every symbol include/*.h declares, and its
argument checks return the statuses that mirror the reference's ArgumentErrors (no compute)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        names |= set(re.findall(r"^STC_API\s+[\w\s\*]+?\b(stc_\w+)\s*\(", h.read_text(), re.M))
    return names


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_abi_version_and_strerror(lib):
    assert lib.stc_abi_version() == 1
    assert b"radius" in lib.stc_strerror(-2)
    assert lib.stc_result_dtype(0, 0, 0) == 0


def _descs(st, abi, stencil, red, bc):
    return abi.LoweredStencil(stencil), abi.lower_op(red), bc


def test_argument_statuses(lib, st, abi):
    src = abi.make_grid(2, abi.F64, (8, 8), (1, 8), 0x1000)
    dst_bad = abi.make_grid(2, abi.F64, (8, 7), (1, 8), 0x2000)
    ls, op, _ = _descs(st, abi, st.Window(1), st.mean, None)
    bc = abi.lower_bc(st.Remove(0.0), st.Conditional())
    # _checksizes: "Source array sizes must match"
    assert lib.stc_map(C.byref(src), C.byref(dst_bad), 0, C.byref(ls.desc), C.byref(op), C.byref(bc), None, 0) == -1
    # radius must be smaller than each axis
    small = abi.make_grid(2, abi.F64, (3, 8), (1, 3), 0x1000)
    small_d = abi.make_grid(2, abi.F64, (3, 8), (1, 3), 0x2000)
    l3 = abi.LoweredStencil(st.Window(3))
    assert lib.stc_map(C.byref(small), C.byref(small_d), 0, C.byref(l3.desc), C.byref(op), C.byref(bc), None, 0) == -2
    # kernelproduct without weights
    kop = abi.lower_op(st.kernelproduct)
    dst = abi.make_grid(2, abi.F64, (8, 8), (1, 8), 0x2000)
    assert lib.stc_map(C.byref(src), C.byref(dst), 0, C.byref(ls.desc), C.byref(kop), C.byref(bc), None, 0) == -3
    # Use with Conditional padding has no method in the reference
    bcu = abi.lower_bc(st.Use(), st.Conditional())
    assert lib.stc_map(C.byref(src), C.byref(dst), 0, C.byref(ls.desc), C.byref(op), C.byref(bcu), None, 0) == -4
    # wrong destination element type
    dst32 = abi.make_grid(2, abi.F32, (8, 8), (1, 8), 0x2000)
    assert lib.stc_map(C.byref(src), C.byref(dst32), 0, C.byref(ls.desc), C.byref(op), C.byref(bc), None, 0) == -4
    # an offset beyond the radius (the Positional all-negative quirk) is rejected
    q = abi.LoweredStencil(st.Positional((-2, -2), (-1, -1)))
    assert lib.stc_map(C.byref(src), C.byref(dst), 0, C.byref(q.desc), C.byref(op), C.byref(bc), None, 0) == -4
    # axis 0 must be contiguous
    strided = abi.make_grid(2, abi.F64, (8, 8), (2, 16), 0x1000)
    assert lib.stc_map(C.byref(strided), C.byref(dst), 0, C.byref(ls.desc), C.byref(op), C.byref(bc), None, 0) == -5
