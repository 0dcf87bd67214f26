"""The registered reductions `f` of `mapstencil(f, A)`.

The reference accepts any Julia function; the GPU path accepts these, each a fixed fold over
the neighbours in offset order (see `stc_opcode` in include/stencil_cuda.h).  Any other callable
raises `NotImplementedError`: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

# ids of stc_opcode in include/stencil_cuda.h
OP_MEAN, OP_SUM, OP_KDOT, OP_MIN, OP_MAX, OP_LIFE, OP_DIFFUSE = range(7)


class Reduction:
    code = -1
    name = "?"

    def __repr__(self):
        return self.name

    def params(self):
        """(birth_mask, survive_mask, alpha) for the stc_op descriptor."""
        return 0, 0, 0.0


class _Mean(Reduction):
    """Statistics.mean over the stencil: left fold of + in offset order, divided by L."""
    code, name = OP_MEAN, "mean"


class _Sum(Reduction):
    """sum over the stencil (StaticArrays' unrolled left fold)."""
    code, name = OP_SUM, "sum"


class _KernelProduct(Reduction):
    """kernelproduct(hood): s = zero; s += hood[i] * kernel[i] (src/stencils/kernel.jl:37-43)."""
    code, name = OP_KDOT, "kernelproduct"


class _Minimum(Reduction):
    code, name = OP_MIN, "minimum"


class _Maximum(Reduction):
    code, name = OP_MAX, "maximum"


mean = _Mean()
sum = _Sum()  # noqa: A001 - mirrors Julia's Base.sum as a registered reduction
kernelproduct = _KernelProduct()
minimum = _Minimum()
maximum = _Maximum()


class LifeRule(Reduction):
    """Outer-totalistic CA rule B{birth}/S{survive} over the count of nonzero neighbours.

    `LifeRule((3,), (2, 3))` is Conway's Life, the closure `s == 3 || (c && s == 2)`.
    """
    code = OP_LIFE

    def __init__(self, birth=(3,), survive=(2, 3)):
        self.birth = tuple(int(b) for b in birth)
        self.survive = tuple(int(s) for s in survive)
        for n in self.birth + self.survive:
            if not 0 <= n <= 31:
                raise ValueError("neighbour counts must be in 0..31")
        self.name = "B" + "".join(map(str, self.birth)) + "/S" + "".join(map(str, self.survive))

    def params(self):
        bm = 0
        for b in self.birth:
            bm |= 1 << b
        sm = 0
        for s in self.survive:
            sm |= 1 << s
        return bm, sm, 0.0


life = LifeRule()


class Diffusion(Reduction):
    """Explicit diffusion step c + alpha * (sum(hood) - L * c), with alpha = dt * D."""
    code = OP_DIFFUSE

    def __init__(self, alpha: float):
        self.alpha = float(alpha)
        self.name = f"diffusion({self.alpha})"

    def params(self):
        return 0, 0, self.alpha


def as_reduction(f) -> Reduction:
    if isinstance(f, Reduction):
        return f
    import builtins
    if f is builtins.sum:
        return sum
    if f is builtins.min:
        return minimum
    if f is builtins.max:
        return maximum
    try:
        import statistics
        if f is statistics.mean:
            return mean
    except ImportError:  # pragma: no cover
        pass
    raise NotImplementedError(
        f"{f!r} is not a registered reduction; the GPU path runs mean, sum, kernelproduct, "
        "minimum, maximum, LifeRule and Diffusion")


# ------------------------------------------------------------------ several arrays
# The reference's multi-array form mapstencil(f, A, B, ...) passes f one stencil per StencilArray
# argument and one value per plain array (src/gatherstencil.jl:105-113).  The registered f is a sum
# of one term per argument, evaluated left to right: Terms(t_1, ..., t_n).

class _Center(Reduction):
    """center(hood): the argument's own value at I."""
    name = "center"


class _Value(Reduction):
    """The value at I of a plain (non-stencil) array argument."""
    name = "value"


center = _Center()
value = _Value()

# ids of stc_term_kind in include/stencil_cuda.h
_TERM_KIND = {"center": 0, "sum": 1, "mean": 2, "kernelproduct": 3, "value": 4}


class Scaled:
    """alpha * term, e.g. `0.1 * sum(neighbors(hood))` (alpha applied in the element type)."""

    def __init__(self, alpha, term):
        if not isinstance(term, Reduction) or term.name not in _TERM_KIND:
            raise NotImplementedError(f"{term!r} is not a registered term")
        self.alpha = float(alpha)
        self.term = term

    def __repr__(self):
        return f"{self.alpha}*{self.term!r}"


def scaled(alpha, term) -> Scaled:
    return Scaled(alpha, term)


class Terms:
    """f(arg_1, ..., arg_n) = t_1 + ... + t_n with t_m one of center, sum, mean, kernelproduct (of
    argument m's stencil) or value (of a plain array), optionally Scaled.  For example the
    reference's `(hood_m, hood_r) -> center(hood_m) + 0.1 * sum(neighbors(hood_r))` is
    `Terms(center, scaled(0.1, sum))`."""

    def __init__(self, *terms):
        used = [t for t in terms if t is not None]
        if not 1 <= len(used) <= 4:
            raise ValueError("1 to 4 terms")
        for t in used:
            base = t.term if isinstance(t, Scaled) else t
            if not isinstance(base, Reduction) or base.name not in _TERM_KIND:
                raise NotImplementedError(f"{t!r} is not a registered term")
        self.terms = terms

    def __repr__(self):
        return " + ".join(repr(t) for t in self.terms if t is not None)

    def lower(self, items, code, grid_fn):
        """TermDesc descriptors for `items`: per argument either a (parent, stencil, boundary, padding)
        tuple or a plain array.  Returns (descs, objects that must outlive the call)."""
        from . import _abi as A
        if len(items) != len(self.terms):
            raise ValueError(f"{len(self.terms)} terms for {len(items)} arguments")
        descs, keep = [], []
        for t, it in zip(self.terms, items):
            if t is None:   # an argument (or layer) the sum does not use
                continue
            base, alpha = (t.term, t.alpha) if isinstance(t, Scaled) else (t, 0.0)
            d = A.TermDesc()
            d.kind = _TERM_KIND[base.name]
            d.scaled = 1 if isinstance(t, Scaled) else 0
            d.alpha = alpha
            if isinstance(it, tuple):
                if base.name == "value":
                    raise TypeError("`value` is the term of a plain array argument")
                parent, stencil, boundary, padding = it
                g = grid_fn(parent)
                ls = A.LoweredStencil(stencil)
                bc = A.lower_bc(boundary, padding, code)
                d.grid = C.pointer(g)
                d.stencil = C.pointer(ls.desc)
                d.bc = C.pointer(bc)
                keep += [g, ls, bc]
            else:
                if base.name != "value":
                    raise TypeError(f"a plain array argument takes the `value` term, not {base.name}")
                g = grid_fn(it)
                d.grid = C.pointer(g)
                keep.append(g)
            descs.append(d)
        return descs, keep
