"""ctypes mirror of include/stencil_cuda.h: the descriptor structs and enum values.

Nothing here touches a GPU; it only lowers host objects (stencils, reductions, boundary flags,
array geometry) into the plain structs the C ABI takes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

STC_OK = 0


class ArgumentError(ValueError):
    """The reference's ArgumentError: mismatched sizes, radius >= axis, kernel length."""

STATUS_NAMES = {
    0: "STC_OK", -1: "STC_ERR_SIZE_MISMATCH", -2: "STC_ERR_RADIUS", -3: "STC_ERR_KERNEL_LENGTH",
    -4: "STC_ERR_UNSUPPORTED", -5: "STC_ERR_INVALID", -6: "STC_ERR_CUDA", -7: "STC_ERR_TIMEOUT",
    -8: "STC_ERR_NO_DEVICE", -9: "STC_ERR_BUDGET", -10: "STC_ERR_BUSY", -11: "STC_ERR_CANCELLED",
    -12: "STC_ERR_TOO_LARGE", -13: "STC_ERR_INEXACT", -14: "STC_ERR_BOUNDS",
}
STC_ERR_BUSY = -10
STC_ASYNC = 1
STC_KEEP_F32 = 2

F64, F32, BF16, F16, U8, BOOL, I32, I64 = range(8)
DTYPE_SIZE = {F64: 8, F32: 4, BF16: 2, F16: 2, U8: 1, BOOL: 1, I32: 4, I64: 8}
FLOAT_DTYPES = (F64, F32, BF16, F16)
DTYPE_NAMES = {F64: "f64", F32: "f32", BF16: "bf16", F16: "f16", U8: "u8", BOOL: "bool",
               I32: "i32", I64: "i64"}

# numpy views of each element type (bf16 is carried as raw uint16 bits on the host)
NP_DTYPE = {F64: np.float64, F32: np.float32, BF16: np.uint16, F16: np.float16, U8: np.uint8,
            BOOL: np.uint8, I32: np.int32, I64: np.int64}


_TORCH_CODES = None


def torch_dtype_code(dt) -> int:
    global _TORCH_CODES
    if _TORCH_CODES is None:
        import torch
        _TORCH_CODES = {torch.float64: F64, torch.float32: F32, torch.bfloat16: BF16, torch.float16: F16,
                        torch.uint8: U8, torch.bool: BOOL, torch.int32: I32, torch.int64: I64}
    code = _TORCH_CODES.get(dt)
    if code is None:
        raise TypeError(f"unsupported element type {dt}")
    return code


def torch_dtype(code: int):
    import torch
    return {F64: torch.float64, F32: torch.float32, BF16: torch.bfloat16, F16: torch.float16,
            U8: torch.uint8, BOOL: torch.bool, I32: torch.int32, I64: torch.int64}[code]


def numpy_dtype_code(dt) -> int:
    dt = np.dtype(dt)
    table = {np.dtype(np.float64): F64, np.dtype(np.float32): F32, np.dtype(np.float16): F16,
             np.dtype(np.uint8): U8, np.dtype(np.bool_): BOOL, np.dtype(np.int32): I32,
             np.dtype(np.int64): I64}
    if dt not in table:
        raise TypeError(f"unsupported element type {dt}")
    return table[dt]


class Grid(C.Structure):
    _fields_ = [("ndims", C.c_int32), ("dtype", C.c_int32), ("size", C.c_int64 * 3),
                ("stride", C.c_int64 * 3), ("data", C.c_void_p)]


class StencilDesc(C.Structure):
    _fields_ = [("ndims", C.c_int32), ("len", C.c_int32), ("radius", C.c_int32), ("shape", C.c_int32),
                ("offsets", C.POINTER(C.c_int32)), ("weights", C.POINTER(C.c_double)),
                ("weight_dtype", C.c_int32), ("reserved", C.c_int32)]


class OpDesc(C.Structure):
    _fields_ = [("code", C.c_int32), ("reserved", C.c_int32), ("birth_mask", C.c_uint32),
                ("survive_mask", C.c_uint32), ("alpha", C.c_double)]


class BcDesc(C.Structure):
    _fields_ = [("boundary", C.c_int32), ("padding", C.c_int32), ("padval", C.c_double),
                ("padval_int", C.c_int64), ("padval_type", C.c_int32), ("reserved", C.c_int32)]


# stc_term_kind
TERM_CENTER, TERM_SUM, TERM_MEAN, TERM_KDOT, TERM_VALUE = range(5)
MAX_TERMS = 4


class TermDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("scaled", C.c_int32), ("alpha", C.c_double),
                ("grid", C.POINTER(Grid)), ("stencil", C.POINTER(StencilDesc)), ("bc", C.POINTER(BcDesc))]


class JobDesc(C.Structure):
    _fields_ = [("grid", Grid), ("stencil", StencilDesc), ("op", OpDesc), ("bc", BcDesc),
                ("nsteps", C.c_int64)]


_PAD_SIZE = ((), (1, 1), (1,), ())
_PAD_STRIDE = ((), (0, 0), (0,), ())


def make_grid(ndims, dtype, size, stride, ptr) -> Grid:
    g = Grid()
    g.ndims = ndims
    g.dtype = dtype
    g.size[:] = tuple(int(x) for x in size[:ndims]) + _PAD_SIZE[ndims]
    g.stride[:] = tuple(int(x) for x in stride[:ndims]) + _PAD_STRIDE[ndims]
    g.data = int(ptr)
    return g


def grid_from_torch(t) -> Grid:
    nd = t.dim()
    if nd < 1 or nd > 3:
        raise ValueError("grids have 1 to 3 dimensions")
    shape, strides = t.shape, t.stride()
    if strides[0] != 1 and shape[0] > 1:
        raise ValueError("axis 0 must be contiguous (column-major, as a Julia Array)")
    g = Grid()
    g.ndims = nd
    g.dtype = torch_dtype_code(t.dtype)
    g.size[:] = tuple(shape) + _PAD_SIZE[nd]
    g.stride[:] = (1,) + tuple(strides[1:]) + _PAD_STRIDE[nd]
    g.data = t.data_ptr()
    return g


def grid_from_numpy(a: np.ndarray, code: int | None = None) -> Grid:
    if a.ndim < 1 or a.ndim > 3:
        raise ValueError("grids have 1 to 3 dimensions")
    es = a.itemsize
    strides = [s // es for s in a.strides]
    if a.shape[0] > 1 and strides[0] != 1:
        raise ValueError("axis 0 must be contiguous (use order='F')")
    strides[0] = 1
    code = numpy_dtype_code(a.dtype) if code is None else code
    return make_grid(a.ndim, code, a.shape, strides, a.ctypes.data)


class LoweredStencil:
    """Keeps the ctypes arrays alive while a StencilDesc points at them."""

    def __init__(self, stencil, grid_ndims: int | None = None):
        from .stencil import Kernel
        offs = stencil.offsets()
        n = stencil.ndims
        self.offsets = (C.c_int32 * (len(offs) * n))(*[c for o in offs for c in o])
        self.weights = None
        wdt = F64
        if isinstance(stencil, Kernel):
            self.weights = (C.c_double * len(offs))(*stencil.weights)
            wdt = F32 if stencil.weight_dtype == "f32" else F64
        d = StencilDesc()
        d.ndims = n
        d.len = len(offs)
        d.radius = stencil.radius
        d.shape = stencil.shape_id
        d.offsets = C.cast(self.offsets, C.POINTER(C.c_int32))
        d.weights = C.cast(self.weights, C.POINTER(C.c_double)) if self.weights is not None else None
        d.weight_dtype = wdt
        self.desc = d


_KERNEL_CLS = None


def lowered_stencil(stencil) -> LoweredStencil:
    """LoweredStencil(stencil), lowered once and kept on the stencil object (a stencil's offsets never
    change); a Kernel, whose weights the caller may still change, is lowered on every call."""
    global _KERNEL_CLS
    if _KERNEL_CLS is None:
        from .stencil import Kernel
        _KERNEL_CLS = Kernel
    if isinstance(stencil, _KERNEL_CLS):
        return LoweredStencil(stencil)
    # the lowering is reused only for the same radius, shape, rank and offsets object (a copy with another
    # radius, as an enclosing Layered stencil makes, is lowered afresh)
    key = (stencil.radius, getattr(stencil, "shape_id", None), stencil.ndims, id(getattr(stencil, "_offsets", None)))
    hit = stencil.__dict__.get("_stc_lowered")
    if hit is not None and hit[0] == key:
        return hit[1]
    ls = LoweredStencil(stencil)
    stencil.__dict__["_stc_lowered"] = (key, ls)
    return ls


def lower_op(red) -> OpDesc:
    o = OpDesc()
    o.code = red.code
    bm, sm, alpha = red.params()
    o.birth_mask = bm
    o.survive_mask = sm
    o.alpha = alpha
    return o


_NP_CODE = {np.dtype(np.float64): F64, np.dtype(np.float32): F32, np.dtype(np.float16): F16,
            np.dtype(np.uint8): U8, np.dtype(np.bool_): BOOL, np.dtype(np.int32): I32, np.dtype(np.int64): I64}


def _fits(pv, code) -> bool:
    """True if the Python number pv is exactly a value of element type `code`."""
    if code in (F64, F32, F16):
        return bool(np.array(pv, dtype=NP_DTYPE[code]).astype(np.float64) == pv) or pv != pv
    if code == BF16:
        f = np.float32(pv)
        return bool(f == pv and (f.view(np.uint32) & 0xFFFF) == 0) or pv != pv
    if isinstance(pv, float) and not float(pv).is_integer():
        return False
    lo, hi = {U8: (0, 255), BOOL: (0, 1), I32: (-2**31, 2**31 - 1), I64: (-2**63, 2**63 - 1)}[code]
    return lo <= int(pv) <= hi


def padval_type_code(pv, grid_code: int | None) -> int:
    """The padval's element type for stc_bc.padval_type (1 + dtype code; 0 = the grid's own type).

    The reference promotes the neighbours to promote_type(eltype, typeof(padval)) (src/gatherstencil.jl:50).
    A numpy scalar carries its type (np.float64(0.0) on a Float32 grid promotes to Float64, as Julia's
    Remove(0.0) does).  A Python bool is Julia's Bool.  A plain Python number has no Julia type: it is
    taken as the grid's element type when it is exactly a value of that type (the reference's default
    Remove(zero(eltype))), else as Julia's Int64 (int) or Float64 (float), so Remove(0.5) on a UInt8 grid
    promotes to Float64 instead of silently becoming 0."""
    if isinstance(pv, (np.generic,)) and np.dtype(type(pv)) in _NP_CODE:
        code = _NP_CODE[np.dtype(type(pv))]
        return 0 if code == grid_code else code + 1
    if grid_code is None or grid_code == BOOL and isinstance(pv, (bool, np.bool_)):
        return 0     # no grid type to compare with: a plain number is taken as the grid's own type
    if isinstance(pv, (bool, np.bool_)):
        return BOOL + 1
    if _fits(pv, grid_code):
        return 0
    return (I64 if isinstance(pv, (int, np.integer)) else F64) + 1


def lower_bc(boundary, padding, grid_code: int | None = None) -> BcDesc:
    """The stc_bc of (boundary, padding); grid_code (the grid's element type) decides whether a plain
    Python padval promotes the neighbours (see padval_type_code)."""
    from .boundary import Remove
    b = BcDesc()
    b.boundary = boundary.code
    b.padding = padding.code
    if isinstance(boundary, Remove):
        pv = boundary.padval
        if pv is None:
            raise ValueError("Remove() without a padval cannot feed a numeric reduction; use Remove(0)")
        b.padval_type = padval_type_code(pv, grid_code)
        if isinstance(pv, (bool, np.bool_)):
            pv = int(pv)
        b.padval = float(pv)
        b.padval_int = int(pv) if float(pv).is_integer() else 0
    return b


_BC_CACHE: dict = {}


def lower_bc_shared(boundary, padding, grid_code: int | None = None) -> BcDesc:
    """lower_bc for the per-call paths, memoised on (boundary kind, padval and its type, padding, element
    type).  The descriptor is shared: callers only pass it by reference to the library, never change it."""
    pv = getattr(boundary, "padval", None)
    key = (boundary.code, type(pv), pv, padding.code, grid_code)
    try:
        b = _BC_CACHE.get(key)
    except TypeError:   # an unhashable padval
        return lower_bc(boundary, padding, grid_code)
    if b is None:
        b = lower_bc(boundary, padding, grid_code)
        if len(_BC_CACHE) < 1024:
            _BC_CACHE[key] = b
    return b
