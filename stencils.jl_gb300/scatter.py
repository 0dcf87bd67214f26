"""scatterstencil_ (the reference's scatterstencil!) with registered value functions and combine ops.

Mirrors src/scatterstencil.jl:36-133.  The reference's `f(hood)` returns one value per stencil offset;
the registered forms are

    ScatterConst(c)   map(_ -> c, neighbors(hood))
    scatter_center    map(_ -> center(hood), neighbors(hood))
    scatter_weighted  center(hood) .* kernel   (a Kernel stencil's weights)

and `op` is `operator.add`, `max` or `min` (Julia's +, max, min).  Every dest cell receives its
contributions in the order of the reference's pass schedule run on one thread, so results are exact.
"""
from __future__ import annotations

import builtins
import ctypes as C
import operator

from . import _abi as A
from . import _lib
from .array import AbstractStencilArray, SwitchingStencilArray
from .boundary import Conditional, Halo

SCATTER_CONST, SCATTER_CENTER, SCATTER_WEIGHTED = 0, 1, 2
COMBINE_ADD, COMBINE_MAX, COMBINE_MIN = 0, 1, 2


class ScatterValue:
    code = -1
    constant = 0.0

    def __repr__(self):
        return self.name


class ScatterConst(ScatterValue):
    """Every offset receives the constant c."""
    code = SCATTER_CONST

    def __init__(self, c):
        self.constant = float(c)
        self.name = f"ScatterConst({c})"


class _ScatterCenter(ScatterValue):
    code, name = SCATTER_CENTER, "scatter_center"


class _ScatterWeighted(ScatterValue):
    code, name = SCATTER_WEIGHTED, "scatter_weighted"


scatter_center = _ScatterCenter()
scatter_weighted = _ScatterWeighted()


def _combine_code(op) -> int:
    if op is operator.add:
        return COMBINE_ADD
    if op is builtins.max:
        return COMBINE_MAX
    if op is builtins.min:
        return COMBINE_MIN
    raise NotImplementedError(f"{op!r} is not a registered scatter combine op (operator.add, max, min)")


class ScatterOpDesc(C.Structure):
    _fields_ = [("value", C.c_int32), ("combine", C.c_int32), ("constant", C.c_double)]


def scatterstencil_(f, op, dest, source=None):
    """scatterstencil!(f, op, dest, source) or scatterstencil!(f, op, A::SwitchingStencilArray).

    For a SwitchingStencilArray the dest parent is zeroed, the source scattered into it, and the
    switched array returned (src/scatterstencil.jl:115-133)."""
    from .gather import _Staged, _grid, _require_device
    if not isinstance(f, ScatterValue):
        raise NotImplementedError(f"{f!r} is not a registered scatter value function")
    d = ScatterOpDesc()
    d.value = f.code
    d.combine = _combine_code(op)
    d.constant = f.constant
    if isinstance(dest, SwitchingStencilArray):
        S = dest
        pad = Halo("in") if isinstance(S.padding, Halo) else Conditional()
        target = S.dest
        target.zero_() if hasattr(target, "zero_") else target.fill(0)
        R = S.radius
        inner = target[tuple(slice(R, s - R) for s in target.shape)] if isinstance(S.padding, Halo) else target
        _scatter(d, S.source, inner, S.stencil, S.boundary, pad, _Staged, _grid, _require_device)
        return S.switch()
    if not isinstance(source, AbstractStencilArray):
        raise TypeError("scatterstencil_(f, op, dest, source) needs a StencilArray source")
    _scatter(d, source.parent, dest, source.stencil, source.boundary, source.padding, _Staged, _grid, _require_device)
    return dest


def _scatter(d, parent, dest, stencil, boundary, padding, _Staged, _grid, _require_device):
    lib = _lib.load()
    lst = A.LoweredStencil(stencil)
    code = A.torch_dtype_code(parent.dtype) if hasattr(parent, "device") else A.numpy_dtype_code(parent.dtype)
    bc = A.lower_bc(boundary, padding, code)
    halo = isinstance(padding, Halo)
    stage = _Staged(parent, dest, writeback=(0, 1) if halo else (1,))
    sp, dp = stage.dev
    _require_device(sp)
    gs, gd = _grid(sp), _grid(dp)
    _lib.check(lib.stc_scatter(C.byref(gs), C.byref(gd), C.byref(lst.desc), C.byref(d), C.byref(bc),
                               _lib.current_stream_handle(), 0), "scatterstencil!")
    stage.done()
