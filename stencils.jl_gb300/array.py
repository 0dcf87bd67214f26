"""StencilArray and SwitchingStencilArray: the reference's array wrappers, holding device parents.

Mirrors src/array.jl.  Arrays are in Julia axis order with axis 0 contiguous (column-major, as a
Julia `Array`); a torch tensor qualifies when `t.stride(0) == 1` (allocate with `colmajor_empty` or
pass `torch.from_numpy(np.asfortranarray(a))`).  Index helpers (`indices`, `neighbors`, `stencil_at`)
take 1-based Julia indices, as the reference does.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np

from . import _abi as A
from ._abi import ArgumentError
from .boundary import Conditional, Halo, Remove, Use, Wrap, Reflect, BoundaryCondition, Padding
from .stencil import Stencil, Window


_TENSOR = None


def _is_torch(x) -> bool:
    global _TENSOR
    if _TENSOR is None:
        try:
            import torch
            _TENSOR = torch.Tensor
        except ImportError:  # pragma: no cover
            _TENSOR = ()
    return isinstance(x, _TENSOR)


def colmajor_empty(shape: Sequence[int], dtype, device="cuda"):
    """An uninitialised torch tensor of `shape` (Julia order) whose axis 0 is contiguous."""
    import torch
    shape = tuple(int(s) for s in shape)
    t = torch.empty(tuple(reversed(shape)), dtype=dtype, device=device)
    return t.permute(*reversed(range(len(shape))))


def colmajor_zeros(shape, dtype, device="cuda"):
    t = colmajor_empty(shape, dtype, device)
    t.zero_()
    return t


def colmajor_like(x, shape=None, dtype=None):
    shape = tuple(x.shape) if shape is None else tuple(shape)
    if _is_torch(x):
        return colmajor_empty(shape, x.dtype if dtype is None else dtype, x.device)
    return np.empty(shape, dtype=x.dtype if dtype is None else dtype, order="F")


def to_device(a, device="cuda"):
    """Copy a numpy array (any order) to a column-major device tensor."""
    import torch
    a = np.asarray(a)
    t = torch.from_numpy(np.asfortranarray(a))
    out = colmajor_empty(a.shape, t.dtype, device)
    out.copy_(t)
    return out


def to_host(t) -> np.ndarray:
    """Device tensor -> numpy array in Fortran order (same Julia indexing)."""
    if _is_torch(t):
        if t.dtype.is_floating_point and t.dtype not in _NP_OK:
            t = t.float()
        return np.asfortranarray(t.detach().cpu().numpy())
    return np.asfortranarray(t)


def _np_ok():
    try:
        import torch
        return {torch.float64, torch.float32, torch.float16}
    except ImportError:  # pragma: no cover
        return set()


_NP_OK = _np_ok()


def _eltype_zero(x):
    if _is_torch(x):
        return False if x.dtype.__str__() == "torch.bool" else (0.0 if x.dtype.is_floating_point else 0)
    kind = np.asarray(x).dtype.kind
    return False if kind == "b" else (0.0 if kind == "f" else 0)


def _check_radius(parent, stencil: Stencil):
    """radius < size along every parent axis (src/array.jl:451-453, :577-580)."""
    for s in parent.shape:
        if not stencil.radius < s:
            raise ArgumentError(f"stencil radius is larger than array axis {s}")


def halo_parent_zeros(shape: Sequence[int], R: int, dtype, device="cuda"):
    """A zeroed column-major tensor of `shape` whose interior rows (axis-0 index R onward) start on
    128-byte lines: a view into a larger buffer, with a few leading elements before index 0 and the
    axis-1 stride rounded up to 128 bytes.  The tiled kernels then stage boxes of it by TMA (which needs
    16-byte row strides) and take the vector-column path (which needs the interior's first column on
    an aligned shared-memory index).  Shape, indexing and contents are those of a plain array."""
    import torch
    shape = tuple(int(s) for s in shape)
    es = torch.empty((), dtype=dtype).element_size()
    line = max(1, 128 // es)
    lead = (-R) % line
    pitch = -(-(lead + shape[0]) // line) * line
    buf = colmajor_zeros((pitch,) + shape[1:], dtype, device)
    return buf[lead:lead + shape[0]]


def pad_array(padding: Padding, stencil: Stencil, parent):
    """Halo(:out) allocates a parent larger by R per side with the array in its interior
    (src/padding.jl:104-110); Conditional and Halo(:in) use the array as is."""
    if isinstance(padding, Halo) and padding.kind == "out":
        R = stencil.radius
        shape = tuple(s + 2 * R for s in parent.shape)
        if _is_torch(parent):
            padded = halo_parent_zeros(shape, R, parent.dtype, parent.device)
        else:
            padded = np.zeros(shape, dtype=parent.dtype, order="F")
        inner = tuple(slice(R, R + s) for s in parent.shape)
        padded[inner] = parent
        return padded
    return parent


class AbstractStencilArray:
    parent = None
    stencil: Stencil
    boundary: BoundaryCondition
    padding: Padding

    @property
    def radius(self) -> int:
        return self.stencil.radius

    @property
    def ndim(self) -> int:
        return self.parent.ndim

    @property
    def shape(self):
        """size(A): the parent's size, less 2R per axis for Halo padding (src/array.jl:470-473)."""
        if isinstance(self.padding, Halo):
            return tuple(s - 2 * self.radius for s in self.parent.shape)
        return tuple(self.parent.shape)

    size = shape

    def _interior(self, parent=None):
        p = self.parent if parent is None else parent
        if isinstance(self.padding, Halo):
            R = self.radius
            return p[tuple(slice(R, s - R) for s in p.shape)]
        return p

    def array(self):
        """The logical array (a view of the parent's interior)."""
        return self._interior()

    # ---- index helpers, 1-based like the reference
    def _bounded(self, J):
        b, s = self.boundary, self.shape
        if isinstance(self.padding, Halo) or isinstance(b, (Remove, Use)):
            return tuple(J)
        out = []
        for i, n in zip(J, s):
            if isinstance(b, Wrap):
                out.append(i + n if i < 1 else (i - n if i > n else i))
            else:  # Reflect
                out.append(2 - i if i < 1 else (2 * n - i if i > n else i))
        return tuple(out)

    def indices(self, I):
        """indices(A, I): neighbour indices with Wrap/Reflect applied (src/array.jl:140-144)."""
        return tuple(self._bounded(J) for J in self.stencil.indices(tuple(I)))

    def neighbors(self, I):
        """neighbors(A, I): neighbour values around the 1-based index I (src/array.jl:68-115); for a
        Layered stencil, one tuple per layer (src/stencils/layered.jl:52-54)."""
        return self._neighbors(self.stencil, I)

    def _neighbors(self, stencil, I):
        from .stencil import Layered
        if isinstance(stencil, Layered):
            return tuple(self._neighbors(l, I) for l in stencil.layers)
        host = to_host(self.parent)
        R = self.radius
        vals = []
        halo = isinstance(self.padding, Halo)
        for J in stencil.indices(tuple(I)):
            if halo:
                vals.append(host[tuple(j - 1 + R for j in J)])
                continue
            inb = all(1 <= j <= n for j, n in zip(J, self.shape))
            if inb:
                vals.append(host[tuple(j - 1 for j in J)])
            elif isinstance(self.boundary, Remove):
                vals.append(self.boundary.padval)
            else:
                vals.append(host[tuple(j - 1 for j in self._bounded(J))])
        return vals

    def center(self, I):
        """center of the stencil at the 1-based index I; for a Layered stencil, one per layer."""
        from .stencil import Layered
        host = to_host(self.parent)
        off = self.radius if isinstance(self.padding, Halo) else 0
        c = host[tuple(i - 1 + off for i in I)]

        def per(st):
            return tuple(per(l) for l in st.layers) if isinstance(st, Layered) else c
        return per(self.stencil)


class StencilArray(AbstractStencilArray):
    """An array with a stencil, a boundary condition and a padding (src/array.jl:441-468)."""

    def __init__(self, A_, stencil: Stencil | None = None, boundary: BoundaryCondition | None = None,
                 padding: Padding | None = None):
        stencil = Window(1, A_.ndim) if stencil is None else stencil
        boundary = Remove(_eltype_zero(A_)) if boundary is None else boundary
        padding = Conditional() if padding is None else padding
        parent = pad_array(padding, stencil, A_)
        _check_radius(parent, stencil)
        self.parent = parent
        self.stencil = stencil
        self.boundary = boundary
        self.padding = padding

    @classmethod
    def from_parent(cls, parent, stencil, boundary, padding):
        obj = cls.__new__(cls)
        _check_radius(parent, stencil)
        obj.parent, obj.stencil, obj.boundary, obj.padding = parent, stencil, boundary, padding
        return obj


class SwitchingStencilArray(AbstractStencilArray):
    """Two parents that swap with every mapstencil_ (src/array.jl:564-611)."""

    def __init__(self, A_, stencil: Stencil | None = None, boundary: BoundaryCondition | None = None,
                 padding: Padding | None = None, *, _dest=None):
        stencil = Window(1, A_.ndim) if stencil is None else stencil
        boundary = Remove(_eltype_zero(A_)) if boundary is None else boundary
        padding = Conditional() if padding is None else padding
        if _dest is None:
            source = pad_array(padding, stencil, A_)
            dest = pad_array(padding, stencil, A_)
            if dest is source:
                dest = dest.clone() if _is_torch(dest) else dest.copy(order="F")
                if _is_torch(source) and dest.stride(0) != 1:
                    d2 = colmajor_like(source)
                    d2.copy_(source)
                    dest = d2
        else:
            source, dest = A_, _dest
            if tuple(source.shape) != tuple(dest.shape):
                raise ArgumentError(f"source and dest arrays must be the same size, got "
                                    f"{tuple(source.shape)} and {tuple(dest.shape)}")
        _check_radius(source, stencil)
        self.source = source
        self.dest = dest
        self.stencil = stencil
        self.boundary = boundary
        self.padding = padding

    @property
    def parent(self):
        return self.source

    def switch(self) -> "SwitchingStencilArray":
        """Swap source and dest in a new wrapper (src/array.jl:610-611)."""
        return SwitchingStencilArray(self.dest, self.stencil, self.boundary, self.padding, _dest=self.source)


def switch(A_: SwitchingStencilArray) -> SwitchingStencilArray:
    return A_.switch()
