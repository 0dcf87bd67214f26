"""mapstencil / mapstencil_ (the reference's mapstencil!) and gatherstencil / gatherstencil_.

Mirrors src/gatherstencil.jl.  Every map runs in libstencilcuda.so on the current CUDA device and
stream; parents held in host memory (numpy) are staged to the device and the results (and, for
Halo padding, the refreshed halo ring) copied back.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi as A
from . import _lib
from .array import (AbstractStencilArray, StencilArray, SwitchingStencilArray, _is_torch, colmajor_empty,
                    to_device)
from .boundary import Conditional, Halo
from .ops import Terms, as_reduction
from .stencil import Layered, Stencil, with_radius


def result_dtype_code(red, src_code: int, stencil, boundary=None, padding=None) -> int:
    """The reference's result type (src/gatherstencil.jl:41-56): f over neighbours of type
    promote_type(eltype, typeof(padval)) for a Remove boundary."""
    lib = _lib.load()
    wdt = A.LoweredStencil(stencil).desc.weight_dtype
    code = src_code
    if boundary is not None:
        bc = A.lower_bc(boundary, padding or Conditional(), src_code)
        code = lib.stc_neighbor_dtype(src_code, C.byref(bc))
        if code < 0:
            _lib.check(code, "mapstencil")
    rc = lib.stc_result_dtype(red.code, code, wdt)
    if rc < 0:
        raise NotImplementedError(f"{red} is not registered for element type {A.DTYPE_NAMES[code]}")
    return rc


def _code_of(x) -> int:
    return A.torch_dtype_code(x.dtype) if _is_torch(x) else A.numpy_dtype_code(x.dtype)


def _grid(x, code=None):
    return A.grid_from_torch(x) if _is_torch(x) else A.grid_from_numpy(x, code)


def _require_device(x):
    if not _is_torch(x) or x.device.type != "cuda":
        raise TypeError("expected a CUDA tensor")


class _Staged:
    """Device copies of host (numpy) parents, written back on exit."""

    def __init__(self, *arrays, writeback=()):
        self.host = arrays
        self.writeback = set(writeback)
        self.dev = []
        for a in arrays:
            if a is None or _is_torch(a):
                self.dev.append(a)
            else:
                self.dev.append(to_device(a))

    def done(self):
        for i, (h, d) in enumerate(zip(self.host, self.dev)):
            if h is not None and not _is_torch(h) and i in self.writeback:
                h[...] = d.cpu().numpy()


def _flags(sync: bool, staged) -> int:
    """STC_ASYNC only when nothing has to be copied back to host memory afterwards."""
    return 0 if (sync or any(h is not None and not _is_torch(h) for h in staged.host)) else 1


def _run_map(red, dest, src: AbstractStencilArray, dst_padded: bool, sync: bool = True):
    lib = _lib.load()
    st = A.lowered_stencil(src.stencil)
    op = A.lower_op(red)
    halo = isinstance(src.padding, Halo)
    stage = _Staged(src.parent, dest, writeback=(0, 1) if halo else (1,))
    sp, dp = stage.dev
    bc = A.lower_bc_shared(src.boundary, src.padding if not isinstance(src, SwitchingStencilArray) else
                           (Halo("in") if isinstance(src.padding, Halo) else src.padding), _code_of(src.parent))
    _require_device(sp)
    gs, gd = _grid(sp), _grid(dp)
    stream = _lib.current_stream_handle()
    _lib.check(lib.stc_map(C.byref(gs), C.byref(gd), int(dst_padded), C.byref(st.desc), C.byref(op), C.byref(bc),
                           stream, _flags(sync, stage)), "mapstencil")
    stage.done()
    return dest


def _new_dest(like, shape, code):
    if _is_torch(like):
        return colmajor_empty(shape, A.torch_dtype(code), like.device)
    if code == A.BF16:
        raise TypeError("bfloat16 results need a device (torch) parent")
    return np.empty(shape, dtype=A.NP_DTYPE[code], order="F")


def _term_items(a):
    """A multi-array argument as oracle-style items: (parent, stencil, boundary, padding) for a
    StencilArray (a SwitchingStencilArray contributes its current source; a Layered stencil one item
    per leaf layer, each with the Layered radius, over the same parent), else the plain array."""
    if isinstance(a, AbstractStencilArray):
        parent = a.source if isinstance(a, SwitchingStencilArray) else a.parent
        if isinstance(a.stencil, Layered):
            R = a.stencil.radius
            return [(parent, with_radius(l, R), a.boundary, a.padding) for l in a.stencil.leaves()]
        return [(parent, a.stencil, a.boundary, a.padding)]
    return [a]



def _run_terms(f: Terms, dest, args, dst_padded: bool, sync: bool = True):
    """dest[I] = f(args at I) through stc_map_terms (src/gatherstencil.jl:89-113)."""
    lib = _lib.load()
    items = [it for a in args for it in _term_items(a)]
    arrays = [it[0] if isinstance(it, tuple) else it for it in items]
    halo_idx = [i for i, it in enumerate(items) if isinstance(it, tuple) and isinstance(it[3], Halo)]
    stage = _Staged(*arrays, dest, writeback=tuple(halo_idx) + (len(arrays),))
    dev = stage.dev
    for d in dev:
        _require_device(d)
    ditems = [(dv,) + it[1:] if isinstance(it, tuple) else dv for it, dv in zip(items, dev[:-1])]
    code = _code_of(dev[0])
    descs, keep = f.lower(ditems, code, _grid)
    gd = _grid(dev[-1])
    arr = (A.TermDesc * len(descs))(*descs)
    _lib.check(lib.stc_map_terms(arr, len(descs), C.byref(gd), int(dst_padded), _lib.current_stream_handle(),
                                 _flags(sync, stage)), "mapstencil")
    del keep
    stage.done()
    return dest


def mapstencil(f, *args, boundary=None, padding=None):
    """mapstencil(f, A::StencilArray, args...) or mapstencil(f, stencil, A; boundary, padding).

    Returns a new array of size(A) holding f applied to the stencil around every cell
    (src/gatherstencil.jl:14-39).  With extra array arguments (the reference's multi-array form) f
    must be a registered `Terms` sum, one term per argument.
    """
    if isinstance(f, Terms):
        sa = args[0]
        if not isinstance(sa, AbstractStencilArray):
            raise TypeError("mapstencil needs a StencilArray first argument")
        dest = _new_dest(sa.parent if not isinstance(sa, SwitchingStencilArray) else sa.source, sa.shape,
                         _code_of(sa.parent if not isinstance(sa, SwitchingStencilArray) else sa.source))
        return _run_terms(f, dest, args, dst_padded=False)
    red = as_reduction(f)
    if args and isinstance(args[0], Stencil):
        hood, arr = args[0], args[1]
        rest = args[2:]
        sa = StencilArray(arr, hood, boundary, padding)
    else:
        sa, rest = args[0], args[1:]
        if not isinstance(sa, AbstractStencilArray):
            raise TypeError("mapstencil needs a StencilArray or (stencil, array)")
    if rest:
        raise NotImplementedError("extra array arguments are not part of the registered GPU path")
    code = result_dtype_code(red, _code_of(sa.parent), sa.stencil, sa.boundary, sa.padding)
    dest = _new_dest(sa.parent, sa.shape, code)
    if isinstance(sa, SwitchingStencilArray):
        sa = StencilArray.from_parent(sa.source, sa.stencil, sa.boundary, sa.padding)
    return _run_map(red, dest, sa, dst_padded=False)


def mapstencil_(f, dest, source=None, *more, steps: int = 1, sync: bool = True, keep_f32: bool = False):
    """mapstencil!(f, dest, source) or mapstencil!(f, A::SwitchingStencilArray).

    For a SwitchingStencilArray, runs `steps` maps (default 1) and returns the switched array, as
    `A = mapstencil!(f, A)` repeated `steps` times would (src/gatherstencil.jl:77-83).  Like the
    reference (KernelAbstractions.synchronize, src/gatherstencil.jl:100) the call waits for the GPU;
    `sync=False` returns once the work is queued on the current CUDA stream (errors a kernel reports
    then surface at the next synchronising call), so consecutive calls keep the GPU busy.

    `keep_f32=True` (BFloat16 / Float16 state of a 3D multi-step run, STC_KEEP_F32) is the precision
    mode: the state stays Float32 inside 4-step passes and is rounded to the 16-bit type at their ends
    (BFloat16 stochastically, from deterministic hashed bits), instead of to nearest after every step.
    """
    if isinstance(f, Terms):
        if isinstance(dest, SwitchingStencilArray):
            # gatherstencil!(f, A::SwitchingStencilArray, B, args...): A's source is the first argument,
            # its dest parent receives the result, then switch(A) (src/gatherstencil.jl:84-88)
            args = (dest,) + ((source,) if source is not None else ()) + tuple(more)
            _run_terms(f, dest.dest, args, dst_padded=isinstance(dest.padding, Halo), sync=sync)
            return dest.switch()
        sa = source
        if not isinstance(sa, AbstractStencilArray):
            raise TypeError("mapstencil_(f, dest, source, args...) needs a StencilArray source")
        padded = tuple(dest.shape) != tuple(sa.shape)
        if padded and not (isinstance(sa.padding, Halo) and tuple(dest.shape) == tuple(sa.parent.shape)):
            raise A.ArgumentError(f"Source array sizes must match. Found: {tuple(sa.shape)} and {tuple(dest.shape)}")
        return _run_terms(f, dest, (sa,) + tuple(more), dst_padded=padded, sync=sync)
    red = as_reduction(f)
    if more:
        raise NotImplementedError("extra array arguments need a registered Terms f")
    if isinstance(dest, SwitchingStencilArray):
        return _run_steps(red, dest, int(steps), sync, keep_f32)
    if not isinstance(source, AbstractStencilArray):
        raise TypeError("mapstencil_(f, dest, source) needs a StencilArray source")
    if tuple(dest.shape) != tuple(source.shape):
        padded = isinstance(source.padding, Halo) and tuple(dest.shape) == tuple(source.parent.shape)
        if not padded:
            raise A.ArgumentError(f"Source array sizes must match. Found: {tuple(source.shape)} and "
                                  f"{tuple(dest.shape)}")
        return _run_map(red, dest, source, dst_padded=True, sync=sync)
    return _run_map(red, dest, source, dst_padded=False, sync=sync)


def _run_steps(red, S: SwitchingStencilArray, steps: int, sync: bool = True,
               keep_f32: bool = False) -> SwitchingStencilArray:
    if steps < 0:
        raise ValueError("steps must be >= 0")
    lib = _lib.load()
    st = A.lowered_stencil(S.stencil)
    op = A.lower_op(red)
    pad = Halo("in") if isinstance(S.padding, Halo) else Conditional()
    bc = A.lower_bc_shared(S.boundary, pad, _code_of(S.source))
    stage = _Staged(S.source, S.dest, writeback=(0, 1))
    a, b = stage.dev
    _require_device(a)
    ga, gb = _grid(a), _grid(b)
    out = C.c_int32(0)
    stream = _lib.current_stream_handle()
    flags = _flags(sync, stage) | (A.STC_KEEP_F32 if keep_f32 else 0)
    _lib.check(lib.stc_map_steps(C.byref(ga), C.byref(gb), C.byref(st.desc), C.byref(op), C.byref(bc), steps,
                                 C.byref(out), stream, flags), "mapstencil!")
    stage.done()
    if out.value:
        return S.switch()
    return S


def update_boundary_(A_: AbstractStencilArray):
    """update_boundary!(A): refresh the halo ring of a Halo-padded parent (src/array.jl:195-233)."""
    if not isinstance(A_.padding, Halo):
        return A_
    lib = _lib.load()
    bc = A.lower_bc(A_.boundary, A_.padding, _code_of(A_.parent))
    stage = _Staged(A_.parent, writeback=(0,))
    g = _grid(stage.dev[0])
    _lib.check(lib.stc_update_boundary(C.byref(g), A_.radius, C.byref(bc), _lib.current_stream_handle(), 0),
               "update_boundary!")
    stage.done()
    return A_


def _host_ptr(host, nbytes: int) -> int:
    if _is_torch(host):
        if host.device.type != "cpu" or not host.is_contiguous():
            raise TypeError("host tensor must be a contiguous CPU tensor")
        ptr, size = host.data_ptr(), host.numel() * host.element_size()
    else:
        a = np.asarray(host)
        if not a.flags.f_contiguous:
            raise TypeError("host array must be column-major contiguous (order='F')")
        ptr, size = a.ctypes.data, a.nbytes
    if size != nbytes:
        raise ValueError(f"host buffer holds {size} bytes, the grid {nbytes}")
    return ptr


def copy_to_device_(dst, host, sync: bool = True):
    """Copy host data into the device grid `dst` (a column-major tensor, or a strided view of one such as
    a Halo parent's interior) as one pitched copy (stc_grid_upload).  `host` is a column-major numpy
    array of dst's size and type, or a contiguous CPU tensor holding the same bytes (pinned memory makes
    the copy asynchronous; with sync=False it must stay valid until the stream reaches the copy)."""
    _require_device(dst)
    lib = _lib.load()
    g = _grid(dst)
    ptr = _host_ptr(host, dst.numel() * dst.element_size())
    _lib.check(lib.stc_grid_upload(C.byref(g), C.c_void_p(ptr), _lib.current_stream_handle(),
                                   0 if sync else A.STC_ASYNC), "copy_to_device_")
    return dst


def copy_to_host_(host, src, sync: bool = True):
    """Copy the device grid `src` (possibly a strided view) into host memory laid out column-major
    (stc_grid_download); the counterpart of copy_to_device_."""
    _require_device(src)
    lib = _lib.load()
    g = _grid(src)
    ptr = _host_ptr(host, src.numel() * src.element_size())
    _lib.check(lib.stc_grid_download(C.c_void_p(ptr), C.byref(g), _lib.current_stream_handle(),
                                     0 if sync else A.STC_ASYNC), "copy_to_host_")
    return host


def mass(x, radius: int = 0, padding=None) -> float:
    """FP64 compensated total of a device grid's logical cells."""
    lib = _lib.load()
    padding = Conditional() if padding is None else padding
    bc = A.BcDesc()
    bc.padding = padding.code
    out = C.c_double(0.0)
    _require_device(x)
    g = _grid(x)
    _lib.check(lib.stc_mass(C.byref(g), radius, C.byref(bc), C.byref(out), _lib.current_stream_handle()), "mass")
    return out.value


gatherstencil = mapstencil
gatherstencil_ = mapstencil_
