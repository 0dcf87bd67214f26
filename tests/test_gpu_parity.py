"""Parity of libstencilcuda.so with the oracle on seeded inputs, and the reference's own goldens
run on the GPU.

Tolerances: every path whose arithmetic follows the reference's order (all Float64 work, every
mean / sum / min / max / diffusion step, integer and Bool work) must be bit-exact.  The one
exception is kernelproduct with Float32 accumulation, which uses fused multiply-adds; it must stay
within 2 * L * 2^-24 * sum|w*v| of the oracle (plus one rounding of the stored half type).
"""
import zlib

import numpy as np
import pytest

import _golden_cases as G
from _backends import GpuBackend, OracleBackend

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(cuda, st, abi):
    return GpuBackend(st, abi)


@pytest.fixture(scope="module")
def ora(st, orc, abi):
    return OracleBackend(st, orc, abi)


@pytest.mark.parametrize("case", G.ALL_CASES, ids=lambda c: c.__name__)
def test_reference_goldens_on_gpu(case, gpu, st, goldens):
    case(gpu, st, goldens)


def test_window_line_equivalence_on_gpu(gpu, st, goldens):
    G.case_window_line_equivalence(gpu, st, goldens, np.random.default_rng(0))


# ------------------------------------------------------------------ seeded parity matrix
def make_input(rng, shape, code, abi, kind="float"):
    if code in (abi.F64, abi.F32, abi.F16):
        dt = {abi.F64: np.float64, abi.F32: np.float32, abi.F16: np.float16}[code]
        a = rng.random(shape).astype(np.float64)
        if kind == "signed":
            a = a * 2 - 1
        return np.asfortranarray(a.astype(dt))
    if code == abi.BF16:
        from oracle.oracle import f32_to_bf16_bits
        a = rng.random(shape).astype(np.float32)
        if kind == "signed":
            a = a * 2 - 1
        return np.asfortranarray(f32_to_bf16_bits(a))
    if code == abi.BOOL or kind == "life":
        bits = (rng.random(shape) < 0.35)
        dt = {abi.U8: np.uint8, abi.BOOL: np.uint8, abi.I32: np.int32, abi.I64: np.int64}[code]
        return np.asfortranarray(bits.astype(dt))
    dt = {abi.U8: np.uint8, abi.I32: np.int32, abi.I64: np.int64}[code]
    return np.asfortranarray(rng.integers(0, 7, size=shape).astype(dt))


def compare(got, want, code_out, abi, tol=None):
    if tol is None:
        if want.dtype.kind == "f":
            ok = np.array_equal(got.view(np.uint64 if want.itemsize == 8 else
                                         (np.uint32 if want.itemsize == 4 else np.uint16)),
                                want.view(np.uint64 if want.itemsize == 8 else
                                          (np.uint32 if want.itemsize == 4 else np.uint16)))
        else:
            ok = np.array_equal(got, want)
        if not ok:
            bad = np.argwhere(got != want)
            raise AssertionError(f"{len(bad)} cells differ; first at {bad[:3].tolist()}: "
                                 f"got {got[tuple(bad[0])]} want {want[tuple(bad[0])]}")
        return
    g = as_f64(got, code_out, abi)
    w = as_f64(want, code_out, abi)
    err = np.abs(g - w)
    assert (err <= tol).all(), f"max excess {np.max(err - tol)}"


def as_f64(x, code, abi):
    if code == abi.BF16:
        from oracle.oracle import bf16_bits_to_f32
        return bf16_bits_to_f32(x).astype(np.float64)
    return x.astype(np.float64)


SHAPES_2D = ["Window1", "Window2", "Window3", "Moore1", "VonNeumann2", "Circle3", "Cross2", "Positional"]


def make_stencil(st, name, nd, rng):
    if name == "Positional":
        offs = set()
        while len(offs) < 6:
            offs.add(tuple(int(x) for x in rng.integers(-2, 3, size=nd)))
        offs = sorted(offs, key=lambda o: rng.random())  # arbitrary order
        offs.append(tuple([2] * nd))                     # radius reaches 2
        return st.Positional(*offs)
    kind, R = name[:-1], int(name[-1])
    return getattr(st, kind)(R, nd)


CASES = []
# (shape name, dims, op, dtype, boundary, padding, size)
for op, dts in (("mean", ["F64", "F32", "BF16", "U8"]), ("sum", ["F64", "F32", "I32", "BOOL"]),
                ("kdot_d", ["F64", "F32", "I64"]), ("kdot_f", ["F32", "BF16", "F16"]),
                ("min", ["F64", "BF16", "I32"]), ("max", ["F32", "U8"]),
                ("life", ["U8", "BOOL", "I32"]), ("diffuse", ["F64", "F32", "BF16"])):
    for dt in dts:
        CASES.append((op, dt))

BOUNDARIES = ["remove0", "remove_nz", "wrap", "reflect"]
PADDINGS = ["cond", "halo_out", "halo_in"]


def _bc(st, name, code, abi):
    if name == "remove0":
        return st.Remove(0)
    if name == "remove_nz":
        if code == abi.BOOL:
            return st.Remove(True)     # a Bool padval: Remove(3) would promote the neighbours to Int64
        return st.Remove(0.75 if code in (abi.F64, abi.F32, abi.BF16, abi.F16) else 3)
    return {"wrap": st.Wrap(), "reflect": st.Reflect()}[name]


def _pad(st, name):
    return {"cond": st.Conditional(), "halo_out": st.Halo("out"), "halo_in": st.Halo("in")}[name]


def _red(st, op):
    return {"mean": st.mean, "sum": st.sum, "kdot_d": st.kernelproduct, "kdot_f": st.kernelproduct,
            "min": st.minimum, "max": st.maximum, "life": st.life, "diffuse": st.Diffusion(0.1)}[op]


def _param_grid():
    out = []
    rng = np.random.default_rng(123)
    sizes2 = [(64, 40), (257, 131), (1000, 37)]
    for (op, dt) in CASES:
        shapes = ["Moore1", "Positional", "VonNeumann2"] if op == "life" else SHAPES_2D
        if op == "diffuse":
            shapes = ["VonNeumann1", "Window1", "Positional"]
        for sh in shapes:
            b = BOUNDARIES[int(rng.integers(len(BOUNDARIES)))]
            p = PADDINGS[int(rng.integers(len(PADDINGS)))]
            size = sizes2[int(rng.integers(len(sizes2)))]
            out.append((op, dt, sh, 2, b, p, size))
    # 3D and 1D
    for (op, dt) in [("mean", "F64"), ("diffuse", "F32"), ("diffuse", "BF16"), ("sum", "I64"), ("life", "U8"),
                     ("kdot_f", "F32"), ("max", "F64")]:
        for sh in ["Moore1", "VonNeumann1", "Cross2", "Positional"]:
            for b in ["remove0", "wrap", "reflect"]:
                out.append((op, dt, sh, 3, b, "cond" if b != "wrap" else "halo_out", (37, 20, 18)))
    for (op, dt) in [("mean", "F64"), ("sum", "F32"), ("kdot_d", "F64")]:
        for b in BOUNDARIES:
            out.append((op, dt, "Window2", 1, b, "cond", (1000,)))
    return out


PARAMS = _param_grid()


@pytest.mark.parametrize("op,dt,shape,nd,bname,pname,size", PARAMS,
                         ids=["-".join(map(str, p[:6])) + "-" + "x".join(map(str, p[6])) for p in PARAMS])
def test_parity_matrix(gpu, ora, st, abi, op, dt, shape, nd, bname, pname, size):
    rng = np.random.default_rng(zlib.crc32(repr((op, dt, shape, nd, bname, pname, size)).encode()))
    code = getattr(abi, dt)
    stencil = make_stencil(st, shape, nd, rng)
    red = _red(st, op)
    if op in ("kdot_d", "kdot_f"):
        w = rng.standard_normal(len(stencil))
        stencil = st.Kernel(stencil, w.astype(np.float32) if op == "kdot_f" else w,
                            weight_dtype="f32" if op == "kdot_f" else "f64")
    bnd = _bc(st, bname, code, abi)
    pad = _pad(st, pname)
    kind = "life" if op == "life" else ("signed" if op in ("min", "max") else "float")
    a = make_input(rng, size, code, abi, kind)
    want = ora.map(a, stencil, red, bnd, pad, code=code)
    got = gpu.map(a, stencil, red, bnd, pad, code=code)
    assert got.shape == want.shape
    out_code = abi.BF16 if (code == abi.BF16 and op not in ("kdot_d",)) else None
    tol = None
    if op == "kdot_f":
        # bound from |w|*|v| through the oracle itself (absolute values, same stencil)
        absk = st.Kernel(stencil.stencil, np.abs(np.array(stencil.weights, dtype=np.float32)), weight_dtype="f32")
        aa = np.abs(as_f64(a, code, abi)).astype(np.float32) if code != abi.F16 else np.abs(a.astype(np.float32))
        mag = ora.map(np.asfortranarray(aa), absk, st.kernelproduct, bnd, pad, code=abi.F32).astype(np.float64)
        L = len(stencil)
        tol = 2 * L * 2.0 ** -24 * mag + 1e-30
        if code in (abi.BF16, abi.F16):
            tol = tol + np.abs(as_f64(want, code, abi)) * (2.0 ** -7 if code == abi.BF16 else 2.0 ** -10) + 1e-6
        compare(got, want, code if code == abi.BF16 else None, abi, tol)
    else:
        compare(got, want, out_code, abi)


def test_specialised_equals_generic(gpu, st, abi):
    """The shape-specialised kernel and the offset-table kernel agree bit for bit."""
    rng = np.random.default_rng(7)
    a = np.asfortranarray(rng.random((517, 263)))
    w1 = st.Window(1)
    as_table = st.Positional(*w1.offsets())
    for bnd in (st.Remove(0.0), st.Wrap(), st.Reflect(), st.Remove(-1.5)):
        x = gpu.map(a, w1, st.mean, bnd, st.Conditional())
        y = gpu.map(a, as_table, st.mean, bnd, st.Conditional())
        assert np.array_equal(x, y)


def test_mean_blur_1000x1000_bit_exact(gpu, ora, st):
    """The config the reference publishes: mapstencil(mean, StencilArray(rand(1000,1000), Window(1)))."""
    a = np.asfortranarray(np.random.default_rng(1).random((1000, 1000)))
    got = gpu.map(a, st.Window(1), st.mean, st.Remove(0.0), st.Conditional())
    want = ora.map(a, st.Window(1), st.mean, st.Remove(0.0), st.Conditional())
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_mean_division_all_binades(gpu, ora, st):
    """Float64 mean of Window(1) (the specialised kernel divides by 9 in integer arithmetic) over values
    spread across every binade, both signs, zeros and subnormals, so that sums land on tiny, huge and
    subnormal quotients (those fall back to the IEEE division): bit-exact against the oracle's
    division, for Window(1) (L = 9) and Window(2) as a table (L = 25, run-time IEEE division)."""
    rng = np.random.default_rng(23)
    shape = (257, 131)
    e = rng.integers(-1074, 1000, size=shape).astype(np.float64)
    a = rng.random(shape) * np.exp2(e) * np.where(rng.random(shape) < 0.5, -1.0, 1.0)
    a[rng.random(shape) < 0.02] = 0.0
    a[rng.random(shape) < 0.02] = 5e-324
    # runs of similar magnitudes, so whole 3x3 blocks share a scale
    blk = np.exp2(rng.integers(-1070, 1000, size=(shape[0] // 8 + 1, shape[1] // 8 + 1)).astype(np.float64))
    a[: shape[0] // 2] = rng.random((shape[0] // 2, shape[1])) * np.kron(blk, np.ones((8, 8)))[: shape[0] // 2, : shape[1]]
    a = np.asfortranarray(a)
    for bnd in (st.Remove(0.0), st.Wrap()):
        for stencil in (st.Window(1), st.Positional(*st.Window(2).offsets())):
            got = gpu.map(a, stencil, st.mean, bnd, st.Conditional())
            want = ora.map(a, stencil, st.mean, bnd, st.Conditional())
            assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (bnd, stencil)


@pytest.mark.parametrize("pad", ["cond", "halo_out"])
@pytest.mark.parametrize("what", ["life", "mean", "diffuse"])
def test_switching_steps_match_oracle(gpu, ora, st, abi, what, pad):
    rng = np.random.default_rng(11)
    padding = _pad(st, pad)
    if what == "life":
        a = np.asfortranarray((rng.random((130, 96)) < 0.3).astype(np.uint8))
        args = (st.Moore(1), st.life, st.Wrap(), padding)
    elif what == "mean":
        a = np.asfortranarray(rng.random((97, 64)))
        args = (st.Window(1), st.mean, st.Remove(0.0), padding)
    else:
        a = np.asfortranarray(rng.random((40, 36, 33)).astype(np.float32))
        args = (st.VonNeumann(1, 3), st.Diffusion(0.1), st.Wrap(), padding)
    for steps in (1, 2, 7):
        got = gpu.switch_map(a, *args, steps=steps)
        want = ora.switch_map(a, *args, steps=steps)
        assert np.array_equal(got, want), (what, steps)


def test_edge_sizes(gpu, ora, st):
    """Grids barely larger than the radius, single rows/columns, and an empty Halo(:in) interior."""
    rng = np.random.default_rng(5)
    for shape in [(2, 2), (4, 3), (3, 200), (200, 3), (2, 1000)]:
        a = np.asfortranarray(rng.random(shape))
        for bnd in (st.Remove(0.0), st.Wrap(), st.Reflect()):
            got = gpu.map(a, st.Window(1), st.mean, bnd, st.Conditional())
            want = ora.map(a, st.Window(1), st.mean, bnd, st.Conditional())
            assert np.array_equal(got, want), (shape, bnd)
    a = np.asfortranarray(rng.random((2, 5)))
    out = gpu.map(a, st.Window(1), st.mean, st.Use(), st.Halo("in"))
    assert out.shape == (0, 3)


def test_argument_errors_on_gpu(cuda, st):
    import torch
    A = st.StencilArray(st.to_device(np.zeros((8, 8))), st.Window(1))
    bad = st.colmajor_empty((8, 7), torch.float64)
    with pytest.raises(st.ArgumentError):
        st.mapstencil_(st.mean, bad, A)


def test_dest_sharing_the_source_memory_is_rejected(cuda, st):
    """mapstencil!(f, dest, A) with dest = A's own parent (or a view into it) has no defined result:
    the library refuses it with STC_ERR_INVALID instead of racing."""
    import torch
    from stencils_gb300._lib import StencilError
    parent = st.to_device(np.asfortranarray(np.random.default_rng(5).random((16, 12))))
    A = st.StencilArray(parent, st.Window(1))
    with pytest.raises(StencilError):
        st.mapstencil_(st.mean, parent, A)
    S = st.SwitchingStencilArray(parent, st.Window(1), st.Wrap(), _dest=parent)
    with pytest.raises(StencilError):
        st.mapstencil_(st.mean, S, steps=2)
    # a separate dest still maps
    out = st.colmajor_empty((16, 12), torch.float64)
    st.mapstencil_(st.mean, out, A)
    torch.cuda.synchronize()
