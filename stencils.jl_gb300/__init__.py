"""stencils_gb300 — Stencils.jl's mapstencil hot path on one GB300 (sm_103a).

The host API mirrors Stencils.jl: stencil shapes (Window, Moore, VonNeumann, Circle, Cross,
Positional, Kernel, ...), boundary conditions (Remove, Wrap, Reflect, Use), padding (Conditional,
Halo), StencilArray / SwitchingStencilArray, and mapstencil / mapstencil_ (the reference's
mapstencil!).  The compute path is libstencilcuda.so (include/stencil_cuda.h), hand-written CUDA
kernels for sm_103a; there is no CPU fallback.
"""
from .array import (AbstractStencilArray, StencilArray, SwitchingStencilArray, colmajor_empty, colmajor_like,
                    colmajor_zeros, switch, to_device, to_host)
from ._abi import ArgumentError
from .batch import Batch
from .boundary import Conditional, Halo, Reflect, Remove, Use, Wrap
from .gather import (copy_to_device_, copy_to_host_, gatherstencil, gatherstencil_, mapstencil, mapstencil_, mass,
                     update_boundary_)
from .ops import Diffusion, LifeRule, Scaled, Terms, center, kernelproduct, life, maximum, mean, minimum, scaled, value
from .ops import sum  # noqa: A004
from .scatter import ScatterConst, scatter_center, scatter_weighted, scatterstencil_
from .serve import Server
from .stencil import (AngledCross, Annulus, BackSlash, Cardinal, Circle, Cross, Diamond, ForwardSlash, Horizontal,
                      Kernel, Layered, Moore, NamedStencil, Ordinal, Positional, Rectangle, Stencil, Vertical,
                      VonNeumann, Window)

__all__ = [
    "Batch", "Server",
    "AbstractStencilArray", "StencilArray", "SwitchingStencilArray", "switch", "colmajor_empty", "colmajor_like",
    "colmajor_zeros", "to_device", "to_host", "ArgumentError", "Conditional", "Halo", "Reflect", "Remove", "Use",
    "Wrap", "gatherstencil", "gatherstencil_", "mapstencil", "mapstencil_", "mass", "update_boundary_",
    "copy_to_device_", "copy_to_host_",
    "Diffusion", "LifeRule", "kernelproduct", "life", "maximum", "mean", "minimum", "sum", "Terms", "Scaled",
    "scaled", "center", "value", "scatterstencil_", "ScatterConst", "scatter_center", "scatter_weighted",
    "AngledCross",
    "Annulus", "BackSlash", "Cardinal", "Circle", "Cross", "Diamond", "ForwardSlash", "Horizontal", "Kernel",
    "Moore", "NamedStencil", "Ordinal", "Positional", "Rectangle", "Stencil", "Vertical", "VonNeumann", "Window",
    "Layered",
]
