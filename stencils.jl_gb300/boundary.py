"""Boundary conditions and padding modes (src/boundary.jl:17-52, src/padding.jl:28-39).

These are flags, as in the reference; the index mapping they imply runs inside the CUDA
kernels' tile loaders (src/array.jl:129-188) and in the halo-fill kernel (src/array.jl:195-239).
"""
from __future__ import annotations

# ids of stc_boundary / stc_padding in include/stencil_cuda.h
REMOVE, WRAP, REFLECT, USE = 0, 1, 2, 3
CONDITIONAL, HALO_IN, HALO_OUT = 0, 1, 2


class BoundaryCondition:
    code = -1

    def __eq__(self, other):
        return type(self) is type(other) and self.__dict__ == other.__dict__

    def __hash__(self):
        return hash((type(self).__name__, tuple(sorted(self.__dict__.items()))))

    def __repr__(self):
        return f"{type(self).__name__}()"


class Wrap(BoundaryCondition):
    """Coordinates past an edge wrap to the opposite side (src/boundary.jl:17)."""
    code = WRAP


class Reflect(BoundaryCondition):
    """Coordinates past an edge mirror back, the edge cell not repeated (src/array.jl:154-166)."""
    code = REFLECT


class Use(BoundaryCondition):
    """Use the existing padding; only valid with Halo padding (src/boundary.jl:42)."""
    code = USE


class Remove(BoundaryCondition):
    """Out-of-bounds neighbours read `padval` (src/boundary.jl:27-32).

    `Remove()` has `padval=None` in the reference (`nothing`); a map over such an array cannot
    produce a numeric result, so the library requires a number.
    """
    code = REMOVE

    def __init__(self, padval=None):
        self.padval = padval

    def __repr__(self):
        return f"Remove({self.padval!r})"


class Padding:
    code = -1

    def __eq__(self, other):
        return type(self) is type(other) and getattr(self, "kind", None) == getattr(other, "kind", None)

    def __hash__(self):
        return hash((type(self).__name__, getattr(self, "kind", None)))


class Conditional(Padding):
    """No halo in memory; the boundary is applied per access (src/padding.jl:39)."""
    code = CONDITIONAL

    def __repr__(self):
        return "Conditional()"


class Halo(Padding):
    """A ring of width R held in memory (src/padding.jl:28-30).

    `Halo(:out)` (the default) allocates a parent larger by R on every side; `Halo(:in)` uses the
    outer ring of the given array, whose logical size is then smaller by 2R.
    """

    def __init__(self, kind: str = "out"):
        kind = kind.lstrip(":")
        if kind not in ("in", "out"):
            raise ValueError("Halo kind must be :in or :out")
        self.kind = kind

    @property
    def code(self):
        return HALO_IN if self.kind == "in" else HALO_OUT

    def __repr__(self):
        return f"Halo(:{self.kind})"
