"""ctypes binding of the CPU oracle (oracle/stencil_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, `__graft_entry__.smoke()` and bench.py's
`cpu_baseline` / `--impl reference` legs, never by the product package.

Arrays are numpy arrays in Julia axis order and column-major memory (`order="F"`); bf16
arrays are carried as uint16 bit patterns.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libstencil_oracle.so"
_lib = None


def build(force: bool = False) -> Path:
    """Compile the oracle with its Makefile (gcc, OpenMP, no FP contraction)."""
    if force or not LIB_PATH.exists() or \
            LIB_PATH.stat().st_mtime < (HERE / "stencil_oracle.c").stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB_PATH))
        from stencils_gb300 import _abi as A  # noqa: F401  (struct layouts)
        P = C.POINTER
        _lib.orc_map.argtypes = [P(A.Grid), P(A.Grid), C.c_int, P(A.StencilDesc), P(A.OpDesc), P(A.BcDesc), C.c_int]
        _lib.orc_map_steps.argtypes = [P(A.Grid), P(A.Grid), P(A.StencilDesc), P(A.OpDesc), P(A.BcDesc),
                                       C.c_int64, C.c_int, P(C.c_int)]
        _lib.orc_update_boundary.argtypes = [P(A.Grid), C.c_int, P(A.BcDesc)]
        _lib.orc_map_terms.argtypes = [P(A.TermDesc), C.c_int, P(A.Grid), C.c_int, C.c_int]
        _lib.orc_scatter.argtypes = [P(A.Grid), P(A.Grid), P(A.StencilDesc), C.c_void_p, P(A.BcDesc), C.c_int]
        _lib.orc_mass.argtypes = [P(A.Grid), C.c_int, C.c_int]
        _lib.orc_mass.restype = C.c_double
        _lib.orc_result_dtype.argtypes = [C.c_int, C.c_int, C.c_int]
        _lib.orc_max_threads.restype = C.c_int
        _lib.orc_f32_to_bf16.argtypes = [C.c_float]
        _lib.orc_f32_to_bf16.restype = C.c_uint16
        _lib.orc_set_fast_paths.argtypes = [C.c_int]
    return _lib


def set_fast_paths(on: bool):
    """Enable (default) or disable the specialised Moore(1) Life path; with it off every map runs the
    generic gather (the tests compare the two)."""
    lib().orc_set_fast_paths(1 if on else 0)


def max_threads() -> int:
    return int(lib().orc_max_threads())


def _check(rc: int, what: str):
    if rc != 0:
        from stencils_gb300._abi import STATUS_NAMES
        raise RuntimeError(f"oracle {what} failed: {STATUS_NAMES.get(rc, rc)}")


def result_dtype(red, src_code: int, weight_code: int = 0) -> int:
    rc = lib().orc_result_dtype(red.code, src_code, weight_code)
    if rc < 0:
        raise NotImplementedError("unsupported (op, dtype) combination")
    return rc


def f32_to_bf16_bits(x: np.ndarray) -> np.ndarray:
    """Round float32 to bfloat16 (nearest even), returned as uint16 bits."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    r[nan] = ((u[nan] >> 16) | 0x40).astype(np.uint16)
    return r.reshape(np.shape(x))


def bf16_bits_to_f32(b: np.ndarray) -> np.ndarray:
    return (np.asarray(b, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def alloc(shape, code: int) -> np.ndarray:
    from stencils_gb300._abi import NP_DTYPE
    return np.zeros(shape, dtype=NP_DTYPE[code], order="F")


def _grid(a: np.ndarray, code: int):
    from stencils_gb300._abi import grid_from_numpy
    return grid_from_numpy(a, code)


# Julia's promote_type over the element types the oracle takes (Bool gives way to anything; an integer and a
# float give the float; integers the wider, UInt8 < Int32 < Int64; floats the wider, BFloat16 with Float16 giving
# Float32), restated here for the padval promotion of src/gatherstencil.jl:50.
def promote_code(a: int, b: int) -> int:
    from stencils_gb300 import _abi as A
    if a == b:
        return a
    if a == A.BOOL:
        return b
    if b == A.BOOL:
        return a
    fa, fb = a in A.FLOAT_DTYPES, b in A.FLOAT_DTYPES
    if fa != fb:
        return a if fa else b
    if not fa:
        rank = {A.U8: 1, A.I32: 2, A.I64: 3}
        return a if rank[a] >= rank[b] else b
    if A.F64 in (a, b):
        return A.F64
    return A.F32


def neighbor_code(src_code: int, boundary) -> int:
    """promote_type(eltype, typeof(padval)) for Remove (src/gatherstencil.jl:41-56, :50), else eltype; the
    padval's type follows the Python layer's lowering rule (stencils_gb300._abi.padval_type_code)."""
    from stencils_gb300 import _abi as A
    from stencils_gb300.boundary import Remove
    if not isinstance(boundary, Remove):
        return src_code
    pt = A.padval_type_code(boundary.padval, src_code)
    return src_code if pt == 0 else promote_code(src_code, pt - 1)


def convert_array(a: np.ndarray, frm: int, to: int) -> np.ndarray:
    """Julia's convert(T, x) elementwise: to a float type round to nearest; to an integer or Bool type the
    value must be exact (else ValueError, the reference's InexactError)."""
    from stencils_gb300 import _abi as A
    if frm == to:
        return np.asfortranarray(a)
    x = bf16_bits_to_f32(a).reshape(a.shape) if frm == A.BF16 else np.asarray(a)
    if to in A.FLOAT_DTYPES:
        if to == A.BF16:
            return np.asfortranarray(f32_to_bf16_bits(x.astype(np.float64).astype(np.float32)))
        return np.asfortranarray(x.astype(A.NP_DTYPE[to]))
    xf = x.astype(np.float64) if x.dtype.kind == "f" else x
    lo, hi = {A.U8: (0, 255), A.BOOL: (0, 1), A.I32: (-2**31, 2**31 - 1), A.I64: (-2**63, 2**63 - 1)}[to]
    if x.dtype.kind == "f" and not np.all(np.isfinite(xf) & (xf == np.trunc(xf))):
        raise ValueError("InexactError: non-integral value")
    if np.any(xf < lo) or np.any(xf > hi):
        raise ValueError("InexactError: value out of range")
    return np.asfortranarray(x.astype(A.NP_DTYPE[to]))


def map(src: np.ndarray, src_code: int, stencil, red, boundary, padding, *,
        dst_code: int | None = None, dst_padded: bool = False, nthreads: int = 1) -> np.ndarray:
    """dst = mapstencil(f, StencilArray(src parent, ...)); updates src's halo like the reference.  A Remove
    padval of another type promotes the neighbours first (the parent converted to the promoted type)."""
    from stencils_gb300 import _abi as A
    ndt = neighbor_code(src_code, boundary)
    if ndt != src_code:
        src, src_code = convert_array(src, src_code, ndt), ndt
    lst = A.LoweredStencil(stencil)
    op = A.lower_op(red)
    bc = A.lower_bc(boundary, padding, src_code)
    if dst_code is None:
        dst_code = result_dtype(red, src_code, lst.desc.weight_dtype)
    R = stencil.radius
    halo = padding.code != 0
    shape = tuple(s - (2 * R if halo else 0) + (2 * R if (halo and dst_padded) else 0) for s in src.shape)
    dst = alloc(shape, dst_code)
    gs, gd = _grid(src, src_code), _grid(dst, dst_code)
    _check(lib().orc_map(C.byref(gs), C.byref(gd), int(dst_padded), C.byref(lst.desc), C.byref(op),
                         C.byref(bc), nthreads), "map")
    return dst


def map_into(src: np.ndarray, src_code: int, dst: np.ndarray, dst_code: int, stencil, red, boundary,
             padding, *, dst_padded: bool = False, nthreads: int = 1):
    from stencils_gb300 import _abi as A
    lst = A.LoweredStencil(stencil)
    op = A.lower_op(red)
    bc = A.lower_bc(boundary, padding, src_code)
    gs, gd = _grid(src, src_code), _grid(dst, dst_code)
    _check(lib().orc_map(C.byref(gs), C.byref(gd), int(dst_padded), C.byref(lst.desc), C.byref(op),
                         C.byref(bc), nthreads), "map")


def map_steps(a: np.ndarray, b: np.ndarray, code: int, stencil, red, boundary, padding, nsteps: int,
              *, nthreads: int = 1) -> bool:
    """nsteps of A = mapstencil!(f, A) on parents (a, b); returns True if b holds the result.  With a
    promoting padval (Conditional padding), every step maps the promoted neighbours and converts the
    result back into the dest parent's type, as the reference's setindex! does."""
    from stencils_gb300 import _abi as A
    ndt = neighbor_code(code, boundary)
    if ndt != code:
        if padding.code != 0:
            raise NotImplementedError("the oracle restates promoted multi-step runs on Conditional grids")
        grids, cur = [a, b], 0
        for _ in range(nsteps):
            y = map(grids[cur], code, stencil, red, boundary, padding, nthreads=nthreads)
            rdt = result_dtype(red, ndt, A.LoweredStencil(stencil).desc.weight_dtype)
            grids[1 - cur][...] = convert_array(y, rdt, code)
            cur = 1 - cur
        return cur == 1
    lst = A.LoweredStencil(stencil)
    op = A.lower_op(red)
    bc = A.lower_bc(boundary, padding, code)
    ga, gb = _grid(a, code), _grid(b, code)
    out = C.c_int(0)
    _check(lib().orc_map_steps(C.byref(ga), C.byref(gb), C.byref(lst.desc), C.byref(op), C.byref(bc),
                               int(nsteps), nthreads, C.byref(out)), "map_steps")
    return bool(out.value)


def _mix32(x: np.ndarray) -> np.ndarray:
    """The "lowbias32" integer hash (Chris Wellons' hash-prospector, public domain), on uint32 arrays."""
    x = x.astype(np.uint32, copy=True)
    x ^= x >> np.uint32(16)
    x *= np.uint32(0x7FEB352D)
    x ^= x >> np.uint32(15)
    x *= np.uint32(0x846CA68B)
    x ^= x >> np.uint32(16)
    return x


def bf16_stochastic_bits(x: np.ndarray, step: int) -> np.ndarray:
    """Float32 (column-major array of the logical grid) -> BFloat16 bits, rounded stochastically: the 16
    bits below the BFloat16 mantissa are added to the magnitude and the sum truncated; the bits are the
    hash of the cell's column-major linear index and `step`.  Infinities and NaN round to nearest."""
    with np.errstate(over="ignore"):
        b = np.asfortranarray(x, dtype=np.float32).ravel(order="F").view(np.uint32)
        lin = np.arange(b.size, dtype=np.uint64)
        s = _mix32(np.array([np.uint32(step) ^ np.uint32(0x9E3779B9)], dtype=np.uint32))[0]
        h = _mix32((lin & np.uint64(0xFFFFFFFF)).astype(np.uint32) ^
                   _mix32((lin >> np.uint64(32)).astype(np.uint32) ^ s))
        special = (b & np.uint32(0x7F800000)) == np.uint32(0x7F800000)
        r = ((b + (h & np.uint32(0xFFFF))) >> np.uint32(16)).astype(np.uint16)
    if special.any():
        r[special] = f32_to_bf16_bits(b[special].view(np.float32))
    return r.reshape(x.shape, order="F")


def keep_f32_schedule(nsteps: int, period: int = 4):
    """The STC_KEEP_F32 precision mode's rounding schedule: m = P * floor((nsteps - 1) / P) steps in passes
    of P (8 for BFloat16, 4 for Float16) held in Float32 and rounded at the end of each pass, then the last
    nsteps - m steps as separate maps (each rounded to nearest).  Returns (passes, per-step tail length)."""
    m = (nsteps - 1) // period * period if nsteps >= 1 else 0
    return m // period, nsteps - m


def map_steps_keep_f32(a: np.ndarray, code: int, stencil, red, boundary, padding, nsteps: int,
                       *, nthreads: int = 1):
    """The STC_KEEP_F32 precision mode restated: 16-bit state `a` (BFloat16 bits or float16).  Each pass
    (8 steps for BFloat16, 4 for Float16) runs as Float32 maps (the oracle's Float32 gather) from the widened state, then rounds (BFloat16
    stochastically with the step number reached, Float16 to nearest); the tail steps are plain 16-bit
    maps.  Returns (state n, state n - 1) as 16-bit arrays of a's type."""
    from stencils_gb300 import _abi as A
    from stencils_gb300.boundary import Remove
    if code == A.BF16:
        widen = bf16_bits_to_f32

        def narrow(x, s):
            return bf16_stochastic_bits(x, s)
    else:
        def widen(x):
            return np.asarray(x, dtype=np.float16).astype(np.float32)

        def narrow(x, s):
            return x.astype(np.float16)
    bnd = boundary
    if isinstance(boundary, Remove):
        # the padval a 16-bit grid's getneighbor returns, widened
        if code == A.BF16:
            pv = widen(f32_to_bf16_bits(np.array([np.float32(boundary.padval)])))
        else:
            pv = np.float32(np.float16(boundary.padval))
        bnd = Remove(float(np.asarray(pv).ravel()[0]))
    period = 8 if code == A.BF16 else 4
    passes, tail = keep_f32_schedule(nsteps, period)
    cur = np.asfortranarray(a)
    prev = cur
    step = 0
    for _ in range(passes):
        pa = np.asfortranarray(widen(cur))
        pb = pa.copy(order="F")
        in_b = map_steps(pa, pb, A.F32, stencil, red, bnd, padding, period, nthreads=nthreads)
        step += period
        prev, cur = cur, np.asfortranarray(narrow(pb if in_b else pa, step))
    if tail:
        pa, pb = cur.copy(order="F"), cur.copy(order="F")
        in_b = map_steps(pa, pb, code, stencil, red, boundary, padding, tail, nthreads=nthreads)
        cur, prev = (pb, pa) if in_b else (pa, pb)
    return cur, prev


def update_boundary(parent: np.ndarray, code: int, radius: int, boundary, padding):
    from stencils_gb300 import _abi as A
    bc = A.lower_bc(boundary, padding)
    g = _grid(parent, code)
    _check(lib().orc_update_boundary(C.byref(g), radius, C.byref(bc)), "update_boundary")


def mass(a: np.ndarray, code: int, radius: int = 0, padding_code: int = 0) -> float:
    g = _grid(a, code)
    return float(lib().orc_mass(C.byref(g), radius, padding_code))


def default_threads() -> int:
    return int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))


def map_terms(f, args, code: int, *, dst_padded: bool = False, nthreads: int = 1) -> np.ndarray:
    """mapstencil(f, args...) for a registered sum of terms `f` (stencils_gb300.Terms).

    `args` are (parent, stencil, boundary, padding) tuples for StencilArray arguments or plain numpy
    arrays; parents are updated in place like the reference's update_boundary!.  Returns the new dest.
    """
    from stencils_gb300 import _abi as A
    descs, keep = f.lower(args, code, lambda a: _grid(a, code))
    first = args[0]
    if isinstance(first, tuple):
        parent, stencil, _, padding = first
        R = stencil.radius if padding.code != 0 else 0
        shape = tuple(s - 2 * R + (2 * R if dst_padded else 0) for s in parent.shape)
    else:
        shape = first.shape
    dst = alloc(shape, code)
    gd = _grid(dst, code)
    arr = (A.TermDesc * len(descs))(*descs)
    _check(lib().orc_map_terms(arr, len(descs), C.byref(gd), int(dst_padded), nthreads), "map_terms")
    del keep
    return dst


def scatter(f, op, dest: np.ndarray, src: np.ndarray, code: int, stencil, boundary, padding, *,
            nthreads: int = 1) -> np.ndarray:
    """scatterstencil!(f, op, dest, StencilArray(src parent, ...)) in place on `dest` (returned)."""
    from stencils_gb300 import _abi as A
    from stencils_gb300.scatter import ScatterOpDesc, _combine_code
    d = ScatterOpDesc()
    d.value = f.code
    d.combine = _combine_code(op)
    d.constant = f.constant
    lst = A.LoweredStencil(stencil)
    bc = A.lower_bc(boundary, padding)
    gs, gd = _grid(src, code), _grid(dest, code)
    _check(lib().orc_scatter(C.byref(gs), C.byref(gd), C.byref(lst.desc), C.byref(d), C.byref(bc), int(nthreads)),
           "scatter")
    return dest
