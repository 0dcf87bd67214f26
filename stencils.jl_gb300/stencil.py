"""Stencil shapes: the offset tables Stencils.jl generates at compile time, restated on the host.

Each shape yields its offsets in exactly the reference's order, component 0 along the
contiguous (column-major first) axis.  The tables are what crosses the C ABI (`stc_stencil`);
shapes with a specialised CUDA kernel also carry a shape id, which the library honours only
when the table matches the shape it specialises.

Reference: src/stencil.jl (abstract Stencil, indices, distances, radius), src/stencils/*.jl.
"""
from __future__ import annotations

import itertools
import math
from typing import Callable, Iterable, Sequence, Tuple

Offset = Tuple[int, ...]

# ids of stc_shape in include/stencil_cuda.h
SHAPE_TABLE, SHAPE_WINDOW, SHAPE_MOORE, SHAPE_VONNEUMANN, SHAPE_CIRCLE, SHAPE_CROSS = range(6)


def _box(R: int, N: int) -> Iterable[Offset]:
    """CartesianIndices(ntuple(_ -> -R:R, N)) in Julia's column-major order (axis 0 fastest)."""
    rng = range(-R, R + 1)
    for rev in itertools.product(rng, repeat=N):
        yield tuple(reversed(rev))


class Stencil:
    """Base of all shapes: `radius`, `ndims`, `offsets`, `len` (src/stencil.jl:17-98)."""

    shape_id = SHAPE_TABLE

    def __init__(self, radius: int, ndims: int, offsets: Sequence[Offset]):
        self.radius = int(radius)
        self.ndims = int(ndims)
        self._offsets = tuple(tuple(int(c) for c in o) for o in offsets)
        if len(self._offsets) == 0:
            raise ValueError("a stencil needs at least one offset")
        for o in self._offsets:
            if len(o) != self.ndims:
                raise ValueError(f"All offsets must be the length `N` of {self.ndims}, got {o}")

    # -- reference API ---------------------------------------------------------------
    def offsets(self) -> Tuple[Offset, ...]:
        return self._offsets

    def __len__(self) -> int:
        return len(self._offsets)

    def diameter(self) -> int:
        return 2 * self.radius + 1

    def distances(self) -> Tuple[float, ...]:
        """sqrt(sum(o^2)) per offset, in Float64 (src/stencil.jl:116-120)."""
        return tuple(math.sqrt(sum(c * c for c in o)) for o in self._offsets)

    def distance_zones(self) -> Tuple[int, ...]:
        return tuple(sum(abs(c) for c in o) for o in self._offsets)

    def indices(self, I: Sequence[int]) -> Tuple[Offset, ...]:
        """Offsets added to I; trailing indices beyond the stencil's N are kept (src/stencil.jl:93-96)."""
        I = tuple(I)
        n = self.ndims
        head, tail = I[:n], I[n:]
        return tuple(tuple(a + b for a, b in zip(o, head)) + tail for o in self._offsets)

    # -- helpers for the C ABI -------------------------------------------------------
    def max_abs_offset(self) -> int:
        return max(max(abs(c) for c in o) for o in self._offsets)

    def is_sorted_colmajor(self) -> bool:
        keys = [tuple(reversed(o)) for o in self._offsets]
        return keys == sorted(keys)

    def __eq__(self, other):
        return (isinstance(other, Stencil) and self.radius == other.radius
                and self.ndims == other.ndims and self._offsets == other._offsets)

    def __hash__(self):
        return hash((self.radius, self.ndims, self._offsets))

    def __repr__(self):
        return f"{type(self).__name__}(radius={self.radius}, ndims={self.ndims}, L={len(self)})"


class _Shape(Stencil):
    """Shapes defined by a predicate over the (2R+1)^N box (the `@stencil` macro, src/stencil.jl:235-277)."""

    def __init__(self, radius: int = 1, ndims: int = 2):
        if radius < 0 or ndims < 1:
            raise ValueError("radius must be >= 0 and ndims >= 1")
        super().__init__(radius, ndims, self._generate(radius, ndims))

    @staticmethod
    def _generate(R: int, N: int):  # pragma: no cover - abstract
        raise NotImplementedError


class Window(_Shape):
    """All cells within radius R, centre included (src/stencils/window.jl:4-7).

    The reference builds its offsets as 2-tuples `(rem(i-1,D)-R, (i-1)÷D-R)` for i in 1:D^N.
    For N=1 `indices` truncates them to their first component; for N>=3 they are wrong (the
    second component runs past R).  Only N<=2 is accepted here.
    """

    shape_id = SHAPE_WINDOW

    @staticmethod
    def _generate(R, N):
        if N > 2:
            raise ValueError("Window offsets are only defined for N <= 2 in the reference "
                             "(src/stencils/window.jl:6); use Moore/Cross/Positional for 3D boxes")
        D = 2 * R + 1
        offs = [((i - 1) % D - R, (i - 1) // D - R) for i in range(1, D ** N + 1)]
        return [o[:N] for o in offs]


class Moore(_Shape):
    """The (2R+1)^N box minus the centre (src/stencils/moore.jl:5-18)."""

    shape_id = SHAPE_MOORE

    @staticmethod
    def _generate(R, N):
        box = list(_box(R, N))
        L = (2 * R + 1) ** N - 1
        return box[: L // 2] + box[L // 2 + 1: L + 1]


class VonNeumann(_Shape):
    """Manhattan distance 1..R (src/stencils/vonneumman.jl:5-15)."""

    shape_id = SHAPE_VONNEUMANN

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N) if 1 <= sum(abs(c) for c in o) <= R]


class Cross(_Shape):
    """Offsets with at least N-1 zero components, centre included (src/stencils/shapes.jl:2-10)."""

    shape_id = SHAPE_CROSS

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N) if sum(1 for c in o if c == 0) >= N - 1]


class AngledCross(_Shape):
    """All diagonals (src/stencils/shapes.jl:13-25)."""

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N) if sum(abs(x) == abs(o[0]) for x in o[1:]) == N - 1]


class ForwardSlash(_Shape):
    """The 'forward' diagonal (src/stencils/shapes.jl:28-40)."""

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N) if sum(x == -o[0] for x in o[1:]) == N - 1]


class BackSlash(_Shape):
    """The 'backward' diagonal (src/stencils/shapes.jl:43-55)."""

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N) if sum(x == o[0] for x in o[1:]) == N - 1]


class Circle(_Shape):
    """Cells whose centre is inside radius R + 0.5 (src/stencils/shapes.jl:58-67)."""

    shape_id = SHAPE_CIRCLE

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N) if math.sqrt(sum(c * c for c in o)) < R + 0.5]


class Vertical(_Shape):
    """A vertical bar or plane (src/stencils/shapes.jl:70-79)."""

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N) if (len(o) > 1 and o[1] == 0) or (len(o) == 1 and o[0] == 0)]


class Horizontal(_Shape):
    """A horizontal bar or plane (src/stencils/shapes.jl:82-91)."""

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N) if len(o) > 1 and o[0] == 0]


class Diamond(_Shape):
    """Manhattan distance 0..R (src/stencils/shapes.jl:94-104)."""

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N) if sum(abs(c) for c in o) <= R]


class Cardinal(_Shape):
    """N/S/E/W points at distance R (src/stencils/shapes.jl:154-163)."""

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N)
                if sum(abs(c) for c in o) == R and max(abs(c) for c in o) == R]


class Ordinal(_Shape):
    """NE/SE/SW/NW corners at distance R (src/stencils/shapes.jl:166-175)."""

    @staticmethod
    def _generate(R, N):
        return [o for o in _box(R, N)
                if sum(abs(c) for c in o) == R * N and max(abs(c) for c in o) == R]


class Annulus(Stencil):
    """A donut: RI + 0.5 <= distance < RO + 0.5 (src/stencils/shapes.jl:116-151); radius is RO."""

    def __init__(self, outer_radius: int = 2, inner_radius: int | None = None, ndims: int = 2):
        RO = int(outer_radius)
        RI = RO - 1 if inner_radius is None else int(inner_radius)
        offs = []
        for o in _box(RO, ndims):
            d = math.sqrt(sum(c * c for c in o))
            if RO + 0.5 > d >= RI + 0.5:
                offs.append(o)
        super().__init__(RO, ndims, offs)


def _positional_radius(offsets: Sequence[Offset]) -> int:
    """`maximum(map(maximum, O))` (src/stencils/positional.jl:74-76).

    This is the reference's radius, NOT the largest absolute offset: a table whose offsets are all
    negative gets too small a radius and the reference's Conditional fast path then reads out of
    bounds.  The library rejects any table whose max-abs offset exceeds the radius.
    """
    return max(max(o) for o in offsets)


class Positional(Stencil):
    """Arbitrary offsets (src/stencils/positional.jl:31-56)."""

    def __init__(self, *offsets):
        if len(offsets) == 1 and isinstance(offsets[0], (tuple, list)) and offsets[0] \
                and isinstance(offsets[0][0], (tuple, list)):
            offsets = tuple(offsets[0])
        offsets = tuple(tuple(o) for o in offsets)
        N = len(offsets[0])
        super().__init__(_positional_radius(offsets), N, offsets)


class Rectangle(Stencil):
    """Per-axis (lo, hi) box (src/stencils/rectangle.jl:13-45); radius is the max-abs bound."""

    def __init__(self, *bounds):
        if len(bounds) == 1 and isinstance(bounds[0][0], (tuple, list)):
            bounds = tuple(bounds[0])
        for b in bounds:
            if len(b) != 2:
                raise ValueError(f"All offset tuples must have length `2`, got {bounds}")
        N = len(bounds)
        R = max(max(abs(c) for c in b) for b in bounds)
        ranges = [range(lo, hi + 1) for lo, hi in bounds]
        offs = [tuple(reversed(rev)) for rev in itertools.product(*reversed(ranges))]
        super().__init__(R, N, offs)


class NamedStencil(Stencil):
    """Offsets with names (src/stencils/named.jl:43-85); the kernel only sees the offset table."""

    def __init__(self, base: Stencil | None = None, names: Sequence[str] | None = None, **named):
        if base is not None:
            offs = base.offsets()
            if names is None:
                names = _default_names(base)
            if len(names) != len(offs):
                raise ValueError("Length of keys must match length of offsets and L parameter")
        else:
            names, offs = tuple(named.keys()), tuple(named.values())
        self.names = tuple(names)
        super().__init__(_positional_radius(offs), len(offs[0]), offs)

    def index(self, name: str) -> int:
        return self.names.index(name)


def _default_names(base: Stencil):
    """Cardinal and Ordinal carry fixed compass names (src/stencils/named.jl:87-88)."""
    if isinstance(base, Cardinal):
        return ("E", "S", "N", "W")
    if isinstance(base, Ordinal):
        return ("SE", "NE", "SW", "NW")
    raise ValueError("names are required for this stencil")


class Kernel(Stencil):
    """A stencil plus weights (src/stencils/kernel.jl:93-116).

    `Kernel(stencil, weights)` takes weights in the stencil's offset order (a column-major
    flattening of an array); `Kernel(f, stencil)` computes `map(f, distances(stencil))`.
    `kernelproduct` is the registered reduction that consumes them.
    """

    def __init__(self, a, b=None, weight_dtype: str | None = None):
        if callable(a) and isinstance(b, Stencil):
            f, hood = a, b
            weights = [f(d) for d in hood.distances()]
        elif isinstance(a, Stencil):
            hood, weights = a, b
        else:
            # Kernel(A::AbstractArray) = Kernel(Window{first(size(A)) ÷ 2, ndims(A)}(), A)
            import numpy as np
            arr = np.asarray(a)
            hood = Window(arr.shape[0] // 2, arr.ndim)
            weights = arr
        import numpy as np
        w = np.asarray(weights)
        if w.ndim > 1:
            w = w.flatten(order="F")
        if len(w) != len(hood):
            raise ValueError(f"Stencil length {len(hood)} does not match kernel length {len(w)}")
        self.stencil = hood
        if weight_dtype is None:
            weight_dtype = "f32" if w.dtype == np.float32 else "f64"
        self.weight_dtype = weight_dtype
        self.weights = tuple(float(x) for x in w)
        self.shape_id = hood.shape_id
        super().__init__(hood.radius, hood.ndims, hood.offsets())


def stencil_radius_ok(st: Stencil) -> bool:
    """True when every offset lies within the radius used for halos and bounds checks."""
    return st.max_abs_offset() <= st.radius


class Layered:
    """Several stencils used together over one array (src/stencils/layered.jl:13-57).

    `Layered(a, b)` or `Layered(name=a, ...)`; layers may themselves be Layered.  The radius is the
    largest layer radius (so a Halo parent is padded for every layer); `offsets`, `indices`,
    `distances`, `len` return one entry per layer, and layers are reached by position or name.
    Maps over a Layered stencil take a registered `Terms` sum with one term per leaf layer (in
    order, nested layers flattened; `None` for a layer the sum does not use): each term reads the
    same parent through its own layer.
    """

    shape_id = SHAPE_TABLE

    def __init__(self, *layers, **named):
        if layers and named:
            raise ValueError("Layered takes positional or named layers, not both")
        if len(layers) == 1 and isinstance(layers[0], (tuple, list)):
            layers = tuple(layers[0])
        self.names = tuple(named) if named else None
        self.layers = tuple(named.values()) if named else tuple(layers)
        if not self.layers:
            raise ValueError("Layered needs at least one layer")
        for l in self.layers:
            if not isinstance(l, (Stencil, Layered)):
                raise TypeError(f"layers must be stencils, got {type(l).__name__}")
        self.ndims = self.layers[0].ndims
        if any(l.ndims != self.ndims for l in self.layers):
            raise ValueError("all layers need the same number of dimensions")
        self.radius = max(l.radius for l in self.layers)

    def __len__(self):
        raise TypeError("length(::Layered) is a tuple: use lengths()")

    def lengths(self):
        return tuple(l.lengths() if isinstance(l, Layered) else len(l) for l in self.layers)

    def __getitem__(self, key):
        if isinstance(key, str):
            return self.layers[self.names.index(key)]
        return self.layers[key]

    def __getattr__(self, name):
        names = self.__dict__.get("names")
        if names and name in names:
            return self.__dict__["layers"][names.index(name)]
        raise AttributeError(name)

    def offsets(self):
        return tuple(l.offsets() for l in self.layers)

    def indices(self, I):
        return tuple(l.indices(I) for l in self.layers)

    def distances(self):
        return tuple(l.distances() for l in self.layers)

    def leaves(self):
        """The leaf stencils in order, nested Layered flattened."""
        out = []
        for l in self.layers:
            out.extend(l.leaves() if isinstance(l, Layered) else [l])
        return out

    def __repr__(self):
        body = ", ".join(f"{n}={l!r}" for n, l in zip(self.names, self.layers)) if self.names else \
            ", ".join(map(repr, self.layers))
        return f"Layered({body})"


def with_radius(stencil: Stencil, R: int) -> Stencil:
    """The same offsets (and weights) with the halo radius R of an enclosing Layered stencil."""
    import copy
    s = copy.copy(stencil)
    s.__dict__.pop("_stc_lowered", None)   # the original's lowering (radius, shape) does not apply
    s.radius = int(R)
    s.shape_id = SHAPE_TABLE
    return s
