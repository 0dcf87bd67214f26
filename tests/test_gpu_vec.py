"""The vector-column map kernels (several adjacent columns per thread, aligned vector loads and stores)
against the oracle, and bit for bit against the one-column kernels they replace.

Every configuration the library registers a vector variant for runs over the four boundaries with
Conditional padding (where the variant applies), on sizes that leave ragged tiles on both axes.
Tolerances are those of the parity matrix: bit-exact, except kernelproduct with Float32 accumulation
(within 2 L 2^-24 sum|w v| of the oracle, plus one rounding of a stored 16-bit type).
"""
import zlib

import numpy as np
import pytest

from _backends import GpuBackend, OracleBackend
from test_gpu_parity import _bc, _red, as_f64, compare, make_input

pytestmark = pytest.mark.gpu

# (op, dtype, shape, R, dims) of each registered vector variant
VEC_CONFIGS = [
    ("kdot_f", "F32", "Window", 3, 2), ("kdot_f", "BF16", "Window", 3, 2), ("kdot_f", "F32", "Window", 2, 2),
    ("mean", "F64", "Window", 1, 2), ("mean", "F32", "Window", 1, 2), ("mean", "BF16", "Window", 1, 2),
    ("mean", "F32", "Circle", 3, 2), ("sum", "F32", "Cross", 2, 2),
    ("life", "U8", "Moore", 1, 2), ("life", "BOOL", "Moore", 1, 2),
    ("diffuse", "F32", "VonNeumann", 1, 3), ("diffuse", "BF16", "VonNeumann", 1, 3),
    ("diffuse", "F64", "VonNeumann", 1, 3),
    ("kdot_f", "F16", "Window", 3, 2), ("mean", "F16", "Window", 1, 2), ("diffuse", "F16", "VonNeumann", 1, 3),
]
BOUNDARIES = ["remove0", "remove_nz", "wrap", "reflect"]


@pytest.fixture(scope="module")
def gpu(cuda, st, abi):
    return GpuBackend(st, abi)


@pytest.fixture(scope="module")
def ora(st, orc, abi):
    return OracleBackend(st, orc, abi)


def _case(st, abi, op, dt, shape, R, nd, size, seed_key):
    rng = np.random.default_rng(zlib.crc32(repr(seed_key).encode()))
    code = getattr(abi, dt)
    stencil = getattr(st, shape)(R, nd)
    if op == "kdot_f":
        stencil = st.Kernel(stencil, rng.standard_normal(len(stencil)).astype(np.float32), weight_dtype="f32")
    kind = "life" if op == "life" else "float"
    return code, stencil, _red(st, op), make_input(rng, size, code, abi, kind)


def _tolerance(st, abi, ora, stencil, a, want, code, bnd, pad):
    absk = st.Kernel(stencil.stencil, np.abs(np.array(stencil.weights, dtype=np.float32)), weight_dtype="f32")
    aa = np.abs(as_f64(a, code, abi)).astype(np.float32)
    mag = ora.map(np.asfortranarray(aa), absk, st.kernelproduct, bnd, pad, code=abi.F32).astype(np.float64)
    tol = 2 * len(stencil) * 2.0 ** -24 * mag + 1e-30
    if code == abi.BF16:
        tol = tol + np.abs(as_f64(want, code, abi)) * 2.0 ** -7 + 1e-6
    if code == abi.F16:
        tol = tol + np.abs(as_f64(want, code, abi)) * 2.0 ** -10 + 1e-7
    return tol


def _sizes(nd):
    return [(131, 70), (517, 263), (9, 300)] if nd == 2 else [(37, 20, 18), (140, 9, 12)]


PARAMS = [(c, b, s) for c in VEC_CONFIGS for b in BOUNDARIES for s in _sizes(c[4])]


@pytest.mark.parametrize("cfg,bname,size", PARAMS,
                         ids=["-".join(map(str, c)) + f"-{b}-" + "x".join(map(str, s)) for c, b, s in PARAMS])
def test_vector_kernel_matches_oracle(gpu, ora, st, abi, cfg, bname, size):
    from stencils_gb300 import _lib
    op, dt, shape, R, nd = cfg
    code, stencil, red, a = _case(st, abi, op, dt, shape, R, nd, size, (cfg, bname, size))
    bnd = _bc(st, bname, code, abi)
    pad = st.Conditional()
    want = ora.map(a, stencil, red, bnd, pad, code=code)
    _lib.profile_enable(True)
    try:
        got = gpu.map(a, stencil, red, bnd, pad, code=code)
        kernels = set(_lib.profile_report())
    finally:
        _lib.profile_enable(False)
    assert any(k.startswith("map_vec") for k in kernels), kernels
    out_code = abi.BF16 if code == abi.BF16 else None
    if op == "kdot_f":
        compare(got, want, out_code, abi, _tolerance(st, abi, ora, stencil, a, want, code, bnd, pad))
    else:
        compare(got, want, out_code, abi)


@pytest.mark.parametrize("cfg", VEC_CONFIGS, ids=["-".join(map(str, c)) for c in VEC_CONFIGS])
def test_vector_kernel_equals_one_column_kernel(gpu, st, abi, monkeypatch, cfg):
    """Same fold order, same operations: the two variants agree bit for bit, Float32 FMAs included."""
    op, dt, shape, R, nd = cfg
    size = (300, 77) if nd == 2 else (70, 21, 19)
    code, stencil, red, a = _case(st, abi, op, dt, shape, R, nd, size, ("eq", cfg))
    for bname in ("remove0", "wrap"):
        bnd = _bc(st, bname, code, abi)
        x = gpu.map(a, stencil, red, bnd, st.Conditional(), code=code)
        monkeypatch.setenv("STC_NO_VEC", "1")
        y = gpu.map(a, stencil, red, bnd, st.Conditional(), code=code)
        monkeypatch.delenv("STC_NO_VEC")
        assert x.dtype == y.dtype and x.tobytes(order="F") == y.tobytes(order="F"), (cfg, bname)


@pytest.mark.parametrize("dt", ["F32", "BF16", "F64"])
@pytest.mark.parametrize("bname", ["wrap", "reflect", "remove_nz"])
@pytest.mark.parametrize("size", [(70, 33, 21), (9, 2, 5), (131, 4, 3), (33, 20, 18), (66, 9, 17)],
                         ids=lambda s: "x".join(map(str, s)))
def test_vector_kernel_padded_multistep(gpu, ora, st, abi, dt, bname, size):
    """3D diffusion over several steps runs on the internal Halo-padded pair (aligned interior rows, so
    its maps take the vector kernel), the ring refreshed between steps; axes of 2 cells and sizes that
    end inside a lane's columns included."""
    code = getattr(abi, dt)
    rng = np.random.default_rng(zlib.crc32(repr((dt, bname, size)).encode()))
    a = make_input(rng, size, code, abi)
    args = (st.VonNeumann(1, 3), st.Diffusion(0.1), _bc(st, bname, code, abi), st.Conditional())
    for steps in (5, 6):
        got = gpu.switch_map(a, *args, steps=steps, code=code)
        want = ora.switch_map(a, *args, steps=steps, code=code)
        assert got.tobytes(order="F") == want.tobytes(order="F"), (dt, bname, size, steps)
