"""scatterstencil! (src/scatterstencil.jl:36-133): the oracle against the reference's own scatter tests
(test/array.jl:385-493), and the GPU (stc_scatter, a deterministic gather) bit for bit against the
oracle, which runs the reference's pass schedule (its delivery order is that of a one-thread run).

The reference's "directional scatter" test needs a two-array value function (water and elevation),
which is not a registered scatter value, so it is not restated here.
"""
import builtins
import operator
import zlib

import numpy as np
import pytest


def _scatter_oracle(st, orc, abi, f, op, src, stencil, boundary=None, padding=None, dest=None):
    boundary = st.Remove(0.0) if boundary is None else boundary
    padding = st.Conditional() if padding is None else padding
    R = stencil.radius
    parent = src
    if isinstance(padding, st.Halo):
        parent = np.zeros(tuple(s + 2 * R for s in src.shape), dtype=src.dtype, order="F")
        parent[R:-R, R:-R] = src
    dest = np.zeros(src.shape, dtype=src.dtype, order="F") if dest is None else dest
    return orc.scatter(f, op, dest, np.asfortranarray(parent), abi.F64 if src.dtype == np.float64 else abi.F32,
                       stencil, boundary, padding)


# ------------------------------------------------------------------ the reference's tests, on the oracle
def test_basic_scatter_add(st, orc, abi):
    """test/array.jl:386-404: each cell scatters 0.1 to its 8 Moore neighbours, Remove(0.0)."""
    d = _scatter_oracle(st, orc, abi, st.ScatterConst(0.1), operator.add, np.ones((5, 5), order="F"), st.Moore(1))
    assert d[2, 2] == pytest.approx(0.8)
    assert d[0, 2] == pytest.approx(0.5) and d[2, 0] == pytest.approx(0.5)
    assert d[0, 0] == pytest.approx(0.3) and d[4, 4] == pytest.approx(0.3)


def test_scatter_max(st, orc, abi):
    """test/array.jl:406-421: each cell scatters its centre value; max keeps the largest."""
    src = np.asfortranarray(np.array([[i + j for j in range(1, 6)] for i in range(1, 6)], dtype=np.float64))
    d = _scatter_oracle(st, orc, abi, st.scatter_center, builtins.max, src, st.Moore(1))
    assert d[2, 2] == 8.0
    assert d[0, 0] == 4.0


def test_vonneumann_scatter(st, orc, abi):
    """test/array.jl:450-465: 0.25 to each VonNeumann(1) neighbour."""
    d = _scatter_oracle(st, orc, abi, st.ScatterConst(0.25), operator.add, np.ones((5, 5), order="F"),
                        st.VonNeumann(1))
    assert d[2, 2] == pytest.approx(1.0)
    assert d[0, 2] == pytest.approx(0.75)
    assert d[0, 0] == pytest.approx(0.5)


def test_larger_radius_scatter(st, orc, abi):
    """test/array.jl:467-478: Moore(2), 0.01 to each of 24 neighbours."""
    d = _scatter_oracle(st, orc, abi, st.ScatterConst(0.01), operator.add, np.ones((7, 7), order="F"), st.Moore(2))
    assert d[3, 3] == pytest.approx(0.24)


def test_scatter_rejects_unregistered(st):
    with pytest.raises(NotImplementedError):
        st.scatterstencil_(lambda h: h, operator.add, np.zeros((3, 3)), None)
    with pytest.raises(NotImplementedError):
        st.scatterstencil_(st.scatter_center, operator.mul, np.zeros((3, 3)), None)


# ------------------------------------------------------------------ GPU against the oracle
VALUES = ["const", "center", "weighted"]
COMBINES = {"add": operator.add, "max": builtins.max, "min": builtins.min}
BOUNDS = ["remove0", "wrap", "reflect", "use"]


def _bc(st, name):
    return {"remove0": st.Remove(0.0), "wrap": st.Wrap(), "reflect": st.Reflect(), "use": st.Use()}[name]


PARAMS = []
for v in VALUES:
    for c in COMBINES:
        for b in BOUNDS:
            pad = "halo" if b == "use" else ("cond" if (len(PARAMS) % 3) else "halo")
            PARAMS.append((v, c, b, pad))


@pytest.mark.gpu
@pytest.mark.parametrize("dt", ["F64", "F32"])
@pytest.mark.parametrize("shape,stencil_name", [((37, 29), "Moore1"), ((20, 11), "Moore2"), ((9, 13), "VonNeumann1")],
                         ids=["37x29-Moore1", "20x11-Moore2", "9x13-VonNeumann1"])
@pytest.mark.parametrize("value,combine,bname,pname", PARAMS, ids=["-".join(p) for p in PARAMS])
def test_scatter_gpu_matches_oracle(cuda, st, orc, abi, dt, shape, stencil_name, value, combine, bname, pname):
    import torch
    rng = np.random.default_rng(zlib.crc32(repr((dt, shape, stencil_name, value, combine, bname, pname)).encode()))
    npdt = np.float64 if dt == "F64" else np.float32
    src = np.asfortranarray((rng.random(shape) * 2 - 1).astype(npdt))
    dest0 = np.asfortranarray((rng.random(shape) * 2 - 1).astype(npdt))
    stencil = getattr(st, stencil_name[:-1])(int(stencil_name[-1]))
    if value == "weighted":
        w = rng.standard_normal(len(stencil))
        stencil = st.Kernel(stencil, w.astype(np.float32) if dt == "F32" else w, weight_dtype="f32" if dt == "F32" else "f64")
    f = {"const": st.ScatterConst(0.3), "center": st.scatter_center, "weighted": st.scatter_weighted}[value]
    op = COMBINES[combine]
    bnd = _bc(st, bname)
    pad = st.Conditional() if pname == "cond" else st.Halo("out")
    want = _scatter_oracle(st, orc, abi, f, op, src, stencil, bnd, pad, dest=dest0.copy(order="F"))
    sa = st.StencilArray(st.to_device(src), stencil, bnd, pad)
    dest = st.to_device(dest0)
    st.scatterstencil_(f, op, dest, sa)
    torch.cuda.synchronize()
    got = st.to_host(dest)
    assert got.tobytes(order="F") == want.tobytes(order="F")


@pytest.mark.gpu
def test_scatter_switching_on_gpu(cuda, st, orc, abi):
    """test/array.jl:480-492 on the GPU: SwitchingStencilArray, 0.1 to each Moore(1) neighbour; the dest
    is cleared first and the switched array returned."""
    import torch
    S = st.SwitchingStencilArray(st.to_device(np.ones((5, 5), order="F")), st.Moore(1), st.Remove(0.0))
    res = st.scatterstencil_(st.ScatterConst(0.1), operator.add, S)
    torch.cuda.synchronize()
    assert res is not S
    out = st.to_host(res.source)
    want = _scatter_oracle(st, orc, abi, st.ScatterConst(0.1), operator.add, np.ones((5, 5), order="F"), st.Moore(1))
    assert out[2, 2] == pytest.approx(0.8)
    assert np.array_equal(out, want)


@pytest.mark.parametrize("bname,nx", [("remove0", 40), ("reflect", 41), ("wrap", 39), ("wrap", 40), ("use", 37)])
def test_threaded_oracle_scatter_equals_one_thread(st, orc, abi, bname, nx):
    """The oracle runs the columns of each pass on threads as the reference does (src/scatterstencil.jl:56-57);
    the result equals the one-thread schedule bit for bit (Wrap with a column count that is not a multiple
    of 2R + 1 runs on one thread)."""
    rng = np.random.default_rng(zlib.crc32(repr(("threads", bname, nx)).encode()))
    for stencil in (st.Moore(1), st.Moore(2), st.VonNeumann(2)):
        src = np.asfortranarray(rng.random((33, nx)) * 2 - 1)
        dest0 = np.asfortranarray(rng.random((33, nx)))
        pad = st.Halo("out") if bname == "use" else st.Conditional()
        one = _scatter_oracle(st, orc, abi, st.scatter_center, operator.add, src, stencil, _bc(st, bname), pad,
                              dest=dest0.copy(order="F"))
        R = stencil.radius
        parent = src
        if bname == "use":
            parent = np.zeros((33 + 2 * R, nx + 2 * R), order="F")
            parent[R:-R, R:-R] = src
        many = orc.scatter(st.scatter_center, operator.add, dest0.copy(order="F"), np.asfortranarray(parent), abi.F64,
                           stencil, _bc(st, bname), pad, nthreads=4)
        assert many.tobytes(order="F") == one.tobytes(order="F")
