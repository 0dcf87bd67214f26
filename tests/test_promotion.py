"""Remove's padval type and the result type it implies (CPU only).

The reference reads the neighbours of a Remove grid as promote_type(eltype, typeof(padval))
(src/gatherstencil.jl:41-56, :50), so `Remove(0.0)` on Float32 yields a Float64 map and `Remove(0.5)` on
UInt8 a Float64 one.  stc_bc carries the padval's type (padval_type); the library's promotion table
(stc_neighbor_dtype) must equal the oracle's restatement of Julia's promote_type, and the Python layer
must lower typed padvals (numpy scalars) and non-representable plain numbers to a promoting padval_type."""
import ctypes as C

import numpy as np
import pytest


def _neighbor(lib, abi, code, boundary):
    bc = abi.lower_bc(boundary, __import__("stencils_gb300").Conditional(), code)
    return lib.stc_neighbor_dtype(code, C.byref(bc))


def test_promotion_table_matches_oracle(lib, abi, orc):
    codes = [abi.F64, abi.F32, abi.BF16, abi.F16, abi.U8, abi.BOOL, abi.I32, abi.I64]
    for a in codes:
        for b in codes:
            bc = abi.BcDesc()
            bc.boundary = 0
            bc.padval_type = b + 1
            assert lib.stc_neighbor_dtype(a, C.byref(bc)) == orc.promote_code(a, b), (a, b)
    bc = abi.BcDesc()
    bc.padval_type = 99
    assert lib.stc_neighbor_dtype(abi.F32, C.byref(bc)) == -5       # malformed padval_type
    bc.boundary = 1                                                # Wrap: no padval, no promotion
    assert lib.stc_neighbor_dtype(abi.F32, C.byref(bc)) == abi.F32


def test_lowering_and_result_types(lib, abi, st):
    from stencils_gb300.gather import result_dtype_code
    # Julia's Remove(0.0) is a Float64 padval: typed here as np.float64
    assert _neighbor(lib, abi, abi.F32, st.Remove(np.float64(0.0))) == abi.F64
    assert result_dtype_code(st.mean, abi.F32, st.Window(1), st.Remove(np.float64(0.0))) == abi.F64
    # a plain Python 0.0 is taken as the grid's own zero (the reference's default Remove(zero(eltype)))
    assert _neighbor(lib, abi, abi.F32, st.Remove(0.0)) == abi.F32
    assert result_dtype_code(st.mean, abi.F32, st.Window(1), st.Remove(0.0)) == abi.F32
    # Remove(0.5) on UInt8: not a UInt8 value, so a Float64 padval (it no longer becomes 0)
    assert _neighbor(lib, abi, abi.U8, st.Remove(0.5)) == abi.F64
    assert result_dtype_code(st.sum, abi.U8, st.Window(1), st.Remove(0.5)) == abi.F64
    assert result_dtype_code(st.mean, abi.U8, st.Window(1), st.Remove(0.5)) == abi.F64
    assert _neighbor(lib, abi, abi.U8, st.Remove(0)) == abi.U8
    assert _neighbor(lib, abi, abi.U8, st.Remove(300)) == abi.I64   # Julia Int
    assert _neighbor(lib, abi, abi.I32, st.Remove(np.int64(7))) == abi.I64
    assert _neighbor(lib, abi, abi.BF16, st.Remove(np.float32(0.5))) == abi.F32
    assert _neighbor(lib, abi, abi.F16, st.Remove(np.float64(0.25))) == abi.F64
    assert _neighbor(lib, abi, abi.BOOL, st.Remove(False)) == abi.BOOL
    assert _neighbor(lib, abi, abi.F32, st.Remove(True)) == abi.F32


def test_oracle_promoted_values(orc, abi, st):
    """A 3x3 UInt8 grid of ones, sum over Window(1) with Remove(0.5): corners 4 + 5 * 0.5, edges 6 + 3 * 0.5,
    the centre 9, all Float64."""
    a = np.ones((3, 3), dtype=np.uint8, order="F")
    got = orc.map(a, abi.U8, st.Window(1), st.sum, st.Remove(0.5), st.Conditional())
    assert got.dtype == np.float64
    want = np.array([[6.5, 7.5, 6.5], [7.5, 9.0, 7.5], [6.5, 7.5, 6.5]])
    assert np.array_equal(got, want)
    # Float32 data with a Float64 padval: the mean runs in Float64 on the widened values
    rng = np.random.default_rng(1)
    x = np.asfortranarray(rng.random((7, 5), dtype=np.float32))
    got = orc.map(x, abi.F32, st.Window(1), st.mean, st.Remove(np.float64(0.1)), st.Conditional())
    ref = orc.map(np.asfortranarray(x.astype(np.float64)), abi.F64, st.Window(1), st.mean, st.Remove(0.1),
                  st.Conditional())
    assert got.dtype == np.float64 and np.array_equal(got, ref)
    # a multi-step run converts each step back to the grid type; a value that does not convert exactly is the
    # reference's InexactError
    pa, pb = np.ones((4, 4), dtype=np.uint8, order="F"), np.ones((4, 4), dtype=np.uint8, order="F")
    with pytest.raises(ValueError):
        orc.map_steps(pa, pb, abi.U8, st.Window(1), st.sum, st.Remove(0.5), st.Conditional(), 1)
