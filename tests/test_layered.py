"""Layered stencils (src/stencils/layered.jl): the reference's Layered test (test/stencils.jl:242-266) on
the host layer, and maps over a Layered stencil with a registered sum of per-layer terms, the GPU bit
for bit against the oracle."""
import zlib

import numpy as np
import pytest


def _ref_layered(st):
    return st.Layered(st.Positional((-1, -1), (1, 1)), st.Positional((-2, -2), (2, 2)))


def test_layered_reference_properties(st):
    """test/stencils.jl:243-253: radius, offsets, indices, neighbors and center of a two-layer stencil."""
    L = _ref_layered(st)
    assert L.radius == 2
    assert L.offsets() == (((-1, -1), (1, 1)), ((-2, -2), (2, 2)))
    assert L.indices((1, 1)) == (((0, 0), (2, 2)), ((-1, -1), (3, 3)))
    A = np.asfortranarray(np.arange(1, 26).reshape(5, 5, order="F"))
    sa = st.StencilArray(A, L)
    assert tuple(tuple(int(x) for x in n) for n in sa.neighbors((3, 3))) == ((7, 19), (1, 25))
    assert tuple(int(c) for c in sa.center((3, 3))) == (13, 13)


def test_nested_named_layers(st):
    """test/stencils.jl:257-262: layers of layers, reached by name."""
    a, b = st.Positional((-1, -1), (1, 1)), st.Positional((-2, -2), (2, 2))
    l1, l2 = st.Layered(a=a, b=b), st.Layered(a=a, b=b)
    ml = st.Layered(l1=l1, l2=l2)
    A = np.asfortranarray(np.arange(1, 26).reshape(5, 5, order="F"))
    sa = st.StencilArray(A, ml)
    filled = sa.neighbors((3, 3))
    assert [int(x) for x in filled[1][0]] == [7, 19]        # ml_filled.l2.a == [7, 19]
    assert ml.l2.a is a and len(ml.leaves()) == 4


def test_layered_map_on_oracle(st, orc, abi):
    """mapstencil(l -> sum(l[1]) - sum(l[2]), StencilArray(A, layered)) (test/stencils.jl:254-256),
    restated as Terms(sum, -1 * sum): a + (-1 * b) == a - b exactly."""
    from stencils_gb300.stencil import with_radius
    L = _ref_layered(st)
    A = np.asfortranarray(np.arange(1, 26).reshape(5, 5, order="F").astype(np.float64))
    items = [(A.copy(order="F"), with_radius(l, L.radius), st.Remove(0.0), st.Conditional()) for l in L.leaves()]
    out = orc.map_terms(st.Terms(st.sum, st.scaled(-1.0, st.sum)), items, abi.F64)
    # cell (3, 3): (7 + 19) - (1 + 25)
    assert out[2, 2] == 0.0
    # cell (1, 1): layer 1 sees (0, 0) -> removed and (2, 2) = 7; layer 2 sees 0 and (3, 3) = 13
    assert out[0, 0] == (0.0 + 7.0) - (0.0 + 13.0)


@pytest.mark.gpu
@pytest.mark.parametrize("dt", ["F64", "F32"])
@pytest.mark.parametrize("bname,pname", [("remove0", "cond"), ("wrap", "cond"), ("reflect", "halo"),
                                          ("wrap", "halo")])
def test_layered_map_gpu_matches_oracle(cuda, st, orc, abi, dt, bname, pname):
    import torch
    from stencils_gb300.stencil import with_radius
    rng = np.random.default_rng(zlib.crc32(repr((dt, bname, pname)).encode()))
    npdt = np.float64 if dt == "F64" else np.float32
    a = np.asfortranarray((rng.random((41, 27)) * 2 - 1).astype(npdt))
    inner = st.Layered(a=st.Moore(1), b=st.Window(2))
    L = st.Layered(x=inner, y=st.Circle(3))            # leaves: Moore(1), Window(2), Circle(3)
    f = st.Terms(st.mean, None, st.scaled(0.5, st.sum))
    bnd = {"remove0": st.Remove(0.0), "wrap": st.Wrap(), "reflect": st.Reflect()}[bname]
    pad = st.Conditional() if pname == "cond" else st.Halo("out")
    R = L.radius
    parent = a
    if pname == "halo":
        parent = np.zeros((a.shape[0] + 2 * R, a.shape[1] + 2 * R), dtype=npdt, order="F")
        parent[R:-R, R:-R] = a
    items = [(parent.copy(order="F"), with_radius(l, R), bnd, pad) for l in L.leaves()]
    want = orc.map_terms(f, items, getattr(abi, dt))
    sa = st.StencilArray.from_parent(st.to_device(parent), L, bnd, pad)
    got = st.to_host(st.mapstencil(f, sa))
    torch.cuda.synchronize()
    assert got.shape == want.shape == a.shape
    assert got.tobytes(order="F") == want.tobytes(order="F")
