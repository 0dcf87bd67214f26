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
    assert lib.stc_abi_version() == 2
    assert b"radius" in lib.stc_strerror(-2)
    assert lib.stc_result_dtype(0, 0, 0) == 0


def _descs(st, abi, stencil, red, bc):
    return abi.LoweredStencil(stencil), abi.lower_op(red), bc


def _no_visible_gpu():
    """The argument tests hand the library placeholder addresses: every call must return from its
    argument checks.  They run only where no GPU is visible, so a call that got past its checks could
    not reach a launch."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("placeholder-address argument tests run only without a visible GPU")


def test_argument_statuses(lib, st, abi):
    _no_visible_gpu()
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


def test_dest_sharing_memory_with_source_is_rejected(lib, st, abi):
    """A dest whose elements share memory with the source has no defined result (tiled reads race the
    writes, as the reference's threads do): every entry point returns STC_ERR_INVALID (-5) before any
    device work."""
    _no_visible_gpu()
    from stencils_gb300.scatter import ScatterOpDesc
    ls, op, _ = _descs(st, abi, st.Window(1), st.mean, None)
    bc = abi.lower_bc(st.Remove(0.0), st.Conditional())
    src = abi.make_grid(2, abi.F64, (8, 8), (1, 8), 0x10000)
    same = abi.make_grid(2, abi.F64, (8, 8), (1, 8), 0x10000)
    shifted = abi.make_grid(2, abi.F64, (8, 8), (1, 8), 0x10000 + 8 * 8 * 8 - 8)   # last element shared
    for dst in (same, shifted):
        assert lib.stc_map(C.byref(src), C.byref(dst), 0, C.byref(ls.desc), C.byref(op), C.byref(bc), None, 0) == -5
        flag = C.c_int32(0)
        assert lib.stc_map_steps(C.byref(src), C.byref(dst), C.byref(ls.desc), C.byref(op), C.byref(bc), 3,
                                 C.byref(flag), None, 0) == -5
        sop = ScatterOpDesc(0, 0, 0.5)
        assert lib.stc_scatter(C.byref(src), C.byref(dst), C.byref(ls.desc), C.byref(sop), C.byref(bc), None, 0) == -5
        term = abi.TermDesc(abi.TERM_SUM, 0, 1.0, C.pointer(src), C.pointer(ls.desc), C.pointer(bc))
        terms = (abi.TermDesc * 1)(term)
        assert lib.stc_map_terms(terms, 1, C.byref(dst), 0, None, 0) == -5


def test_disjoint_views_pass_the_overlap_rule(lib, st, abi):
    """Disjoint grids pass every argument check: the first device step then reports that no GPU is
    visible (STC_ERR_NO_DEVICE, -8) rather than STC_ERR_INVALID.  Adjacent buffers, and two column
    blocks of one wider parent, are disjoint."""
    _no_visible_gpu()
    ls, op, _ = _descs(st, abi, st.Window(1), st.mean, None)
    bc = abi.lower_bc(st.Remove(0.0), st.Conditional())
    src = abi.make_grid(2, abi.F64, (8, 8), (1, 8), 0x10000)
    adjacent = abi.make_grid(2, abi.F64, (8, 8), (1, 8), 0x10000 + 8 * 8 * 8)
    assert lib.stc_map(C.byref(src), C.byref(adjacent), 0, C.byref(ls.desc), C.byref(op), C.byref(bc), None, 0) == -8
    left = abi.make_grid(2, abi.F64, (8, 4), (1, 8), 0x10000)
    right = abi.make_grid(2, abi.F64, (8, 4), (1, 8), 0x10000 + 4 * 8 * 8)
    assert lib.stc_map(C.byref(left), C.byref(right), 0, C.byref(ls.desc), C.byref(op), C.byref(bc), None, 0) == -8
