"""Maps over several arrays, mapstencil(f, A, B, ...) with f a registered sum of terms
(src/gatherstencil.jl:84-113): the oracle against the reference's own multi-array tests
(test/array.jl:312-383), and the GPU (stc_map_terms) bit for bit against the oracle.

All these sums run in the element type with every operation rounded, in the reference's left-to-right
order, so parity is exact.
"""
import zlib

import numpy as np
import pytest

from _backends import GpuBackend


# ------------------------------------------------------------------ the reference's tests, on the oracle
def test_two_stencil_arrays_centers(st, orc, abi):
    """test/array.jl:313-324: center(hood_a) + center(hood_b) == A .+ B."""
    A = np.asfortranarray(np.array([[1, 2, 3], [4, 5, 6], [7, 8, 9]], dtype=np.float64))
    B = np.asfortranarray(np.array([[10, 20, 30], [40, 50, 60], [70, 80, 90]], dtype=np.float64))
    f = st.Terms(st.center, st.center)
    args = [(A.copy(order="F"), st.Moore(1), st.Remove(0.0), st.Conditional()),
            (B.copy(order="F"), st.Moore(1), st.Remove(0.0), st.Conditional())]
    assert np.array_equal(orc.map_terms(f, args, abi.F64), A + B)


def test_two_stencil_arrays_neighbour_sums(st, orc, abi):
    """test/array.jl:326-330: sum(neighbors(hood_a)) + sum(neighbors(hood_b)) has size(A)."""
    A = np.asfortranarray(np.arange(1.0, 10.0).reshape(3, 3))
    B = 10 * A
    f = st.Terms(st.sum, st.sum)
    out = orc.map_terms(f, [(A.copy(order="F"), st.Moore(1), st.Remove(0.0), st.Conditional()),
                            (np.asfortranarray(B), st.Moore(1), st.Remove(0.0), st.Conditional())], abi.F64)
    assert out.shape == A.shape
    # centre cell: every other cell of each 3x3 array
    assert out[1, 1] == (A.sum() - A[1, 1]) + (B.sum() - B[1, 1])


def test_switching_with_stencil_array(st, orc, abi):
    """test/array.jl:333-353: three steps of c + 0.1 * sum(neighbors(hood_r)) grow the centre."""
    mutable = np.asfortranarray(np.array([[0, 0, 0], [0, 1, 0], [0, 0, 0]], dtype=np.float64))
    readonly = np.asfortranarray(np.array([[1, 1, 1], [1, 0, 1], [1, 1, 1]], dtype=np.float64))
    f = st.Terms(st.center, st.scaled(0.1, st.sum))
    cur = mutable.copy(order="F")
    for _ in range(3):
        cur = orc.map_terms(f, [(cur, st.Moore(1), st.Remove(0.0), st.Conditional()),
                                (readonly.copy(order="F"), st.Moore(1), st.Remove(0.0), st.Conditional())], abi.F64)
    assert cur.shape == mutable.shape
    assert cur[1, 1] > mutable[1, 1]
    x = 1.0
    for _ in range(3):
        x = x + 0.1 * 8.0
    assert cur[1, 1] == x


def test_three_stencil_arrays(st, orc, abi):
    """test/array.jl:355-369: center(a) + center(b) + center(c) == 6 on the interior."""
    A, B, C = np.ones((5, 5), order="F"), 2 * np.ones((5, 5), order="F"), 3 * np.ones((5, 5), order="F")
    f = st.Terms(st.center, st.center, st.center)
    out = orc.map_terms(f, [(np.asfortranarray(a), st.Moore(1), st.Remove(0.0), st.Conditional()) for a in (A, B, C)],
                        abi.F64)
    assert np.all(out[1:4, 1:4] == 6.0)


def test_mixed_stencil_and_plain_array(st, orc, abi):
    """test/array.jl:371-382: center(hood_a) + b_val == A .+ B (B a plain array)."""
    A = np.asfortranarray(np.array([[1, 2, 3], [4, 5, 6], [7, 8, 9]], dtype=np.float64))
    B = np.asfortranarray(np.array([[10, 20, 30], [40, 50, 60], [70, 80, 90]], dtype=np.float64))
    f = st.Terms(st.center, st.value)
    out = orc.map_terms(f, [(A.copy(order="F"), st.Moore(1), st.Remove(0.0), st.Conditional()), B], abi.F64)
    assert np.array_equal(out, A + B)


def test_terms_reject_bad_arguments(st):
    with pytest.raises(NotImplementedError):
        st.Terms(st.minimum)
    with pytest.raises(ValueError):
        st.Terms()


# ------------------------------------------------------------------ GPU against the oracle
@pytest.fixture(scope="module")
def gpu(cuda, st, abi):
    return GpuBackend(st, abi)


def _gpu_terms(st, f, items, code):
    """Run mapstencil(f, args...) on the GPU with device copies of the items."""
    import torch
    args = []
    for it in items:
        if isinstance(it, tuple):
            parent, stencil, bnd, pad = it
            d = st.to_device(parent)
            args.append(st.StencilArray.from_parent(d, stencil, bnd, pad))
        else:
            args.append(st.to_device(it))
    out = st.mapstencil(f, *args)
    torch.cuda.synchronize()
    return st.to_host(out)


def _padded(a, R, pad, st):
    if isinstance(pad, st.Halo):
        p = np.zeros(tuple(s + 2 * R for s in a.shape), dtype=a.dtype, order="F")
        p[tuple(slice(R, R + s) for s in a.shape)] = a
        return p
    return np.asfortranarray(a.copy())


CASES = [
    # (terms, per-argument (kind, stencil name, boundary, padding) or "plain")
    ("center+center", [("center", "Moore1", "remove0", "cond"), ("center", "Moore1", "wrap", "cond")]),
    ("sum+sum", [("sum", "Moore1", "remove0", "cond"), ("sum", "Window2", "wrap", "halo")]),
    ("center+0.1sum", [("center", "Moore1", "remove0", "cond"), ("0.1sum", "Moore1", "reflect", "cond")]),
    ("mean+value", [("mean", "Circle2", "wrap", "cond"), "plain"]),
    ("kdot+center+value", [("kdot", "Window1", "remove_nz", "cond"), ("center", "VonNeumann1", "wrap", "halo"),
                           "plain"]),
    ("0.5mean+2center+sum+value", [("0.5mean", "Moore1", "reflect", "halo"), ("2center", "Moore1", "wrap", "cond"),
                                   ("sum", "Cross2", "remove0", "cond"), "plain"]),
]


def _build_case(st, abi, case, shape, dt, seed):
    rng = np.random.default_rng(seed)
    npdt = np.float64 if dt == "F64" else np.float32
    terms, items = [], []
    for spec in case:
        a = rng.random(shape).astype(npdt) * 2 - 1
        a = np.asfortranarray(a.astype(npdt))
        if spec == "plain":
            terms.append(st.value)
            items.append(a)
            continue
        kind, sname, bname, pname = spec
        nd = len(shape)
        kind_name = sname[:-1]
        R = int(sname[-1])
        if nd == 3 and kind_name in ("Window", "Circle"):   # 2D-only generators in the reference; a 3D
            kind_name, R = "Moore", 1                       # term holds at most STC_MAX_TERM_LEN offsets
        stencil = getattr(st, kind_name)(R, nd)
        scale = None
        for k in ("center", "sum", "mean", "kdot"):
            if kind.endswith(k):
                pre = kind[: -len(k)]
                scale = float(pre) if pre else None
                base = {"center": st.center, "sum": st.sum, "mean": st.mean, "kdot": st.kernelproduct}[k]
                if k == "kdot":
                    w = rng.standard_normal(len(stencil))
                    stencil = st.Kernel(stencil, w.astype(np.float32) if dt == "F32" else w,
                                        weight_dtype="f32" if dt == "F32" else "f64")
        terms.append(st.scaled(scale, base) if scale is not None else base)
        bnd = {"remove0": st.Remove(0.0), "remove_nz": st.Remove(0.75), "wrap": st.Wrap(),
               "reflect": st.Reflect()}[bname]
        pad = {"cond": st.Conditional(), "halo": st.Halo("out")}[pname]
        items.append((_padded(a, stencil.radius, pad, st), stencil, bnd, pad))
    return st.Terms(*terms), items


@pytest.mark.gpu
@pytest.mark.parametrize("dt", ["F64", "F32"])
@pytest.mark.parametrize("shape", [(37, 29), (130, 7), (21, 17, 9)], ids=lambda s: "x".join(map(str, s)))
@pytest.mark.parametrize("name,case", CASES, ids=[c[0] for c in CASES])
def test_terms_gpu_matches_oracle(gpu, st, orc, abi, dt, shape, name, case):
    seed = zlib.crc32(repr((name, dt, shape)).encode())
    f, items = _build_case(st, abi, case, shape, dt, seed)
    code = getattr(abi, dt)
    want = orc.map_terms(f, [(it[0].copy(order="F"),) + it[1:] if isinstance(it, tuple) else it for it in items],
                         code)
    got = _gpu_terms(st, f, items, code)
    assert got.shape == want.shape
    assert got.tobytes(order="F") == want.tobytes(order="F"), (name, dt, shape)


@pytest.mark.gpu
def test_terms_switching_form_on_gpu(gpu, st, orc, abi):
    """mapstencil!(f, S::SwitchingStencilArray, B::StencilArray) writes S's dest and switches
    (src/gatherstencil.jl:84-88); three steps equal three oracle maps."""
    import torch
    rng = np.random.default_rng(3)
    m = np.asfortranarray(rng.random((33, 21)))
    r = np.asfortranarray(rng.random((33, 21)))
    f = st.Terms(st.center, st.scaled(0.1, st.sum))
    S = st.SwitchingStencilArray(st.to_device(m), st.Moore(1), st.Remove(0.0))
    B = st.StencilArray(st.to_device(r), st.Moore(1), st.Remove(0.0))
    cur = m.copy(order="F")
    for _ in range(3):
        S = st.mapstencil_(f, S, B)
        cur = orc.map_terms(f, [(cur, st.Moore(1), st.Remove(0.0), st.Conditional()),
                                (r.copy(order="F"), st.Moore(1), st.Remove(0.0), st.Conditional())], abi.F64)
    torch.cuda.synchronize()
    assert np.array_equal(st.to_host(S.source).view(np.uint64), cur.view(np.uint64))


@pytest.mark.gpu
def test_terms_too_long_a_stencil_is_unsupported(gpu, st):
    """A term's stencil holds at most STC_MAX_TERM_LEN (64) offsets."""
    a = st.StencilArray(st.to_device(np.zeros((9, 9, 9))), st.Moore(2, 3))
    with pytest.raises(NotImplementedError):
        st.mapstencil(st.Terms(st.sum), a)


@pytest.mark.gpu
def test_terms_size_mismatch_on_gpu(gpu, st):
    import torch
    a = st.StencilArray(st.to_device(np.zeros((8, 8))), st.Moore(1))
    b = st.to_device(np.zeros((8, 9)))
    with pytest.raises(st.ArgumentError):
        st.mapstencil(st.Terms(st.center, st.value), a, b)
    torch.cuda.synchronize()
