"""The registered reductions `f` of `mapstencil(f, A)`.

The reference accepts any Julia function; the GPU path accepts these, each a fixed fold over
the neighbours in offset order (see `stc_opcode` in include/stencil_cuda.h).  Any other callable
raises `NotImplementedError`: there is no CPU fallback.
"""
from __future__ import annotations

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
    """kernelproduct(hood): s = zero; s += hood[i] * kernel[i] (src/stencils/kernel.jl:264-270)."""
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
