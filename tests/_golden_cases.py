"""The reference's mapstencil test cases (test/array.jl, test/stencils.jl), written once against a
backend (oracle or GPU).  Each function mirrors one reference testset and cites its lines."""
from __future__ import annotations

import numpy as np

RTOL = 1.4901161193847656e-08   # Julia's isapprox default: sqrt(eps(Float64))


def approx(a, b):
    return np.allclose(np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64), rtol=RTOL, atol=0)


def same(*xs):
    """Julia `==` on Float64 arrays, compared bit for bit (no NaNs here)."""
    x0 = np.asarray(xs[0])
    return all(np.array_equal(x0, np.asarray(x)) for x in xs[1:])


def r_5x6():
    i = np.arange(1.0, 6.0)[:, None]
    j = np.arange(100.0, 106.0)[None, :]
    return np.asfortranarray(i * j)                       # (1.0:5.0) * (100.0:105.0)'


def mat(g, name):
    return np.asfortranarray(np.array(g[name]["data"], dtype=np.float64))


def case_remove_use(B, st, g):
    """test/array.jl:123-162 (Remove / Use)."""
    r = r_5x6()
    W = st.Window(1, 2)
    rm = st.Remove(0.0)
    A1 = B.map(r, W, st.mean, rm, st.Conditional())
    B1 = B.map(r, W, st.mean, rm, st.Halo("out"))
    C1 = B.map(r, W, st.mean, st.Use(), st.Halo("in"))
    SA1 = B.switch_map(r, W, st.mean, rm, st.Conditional())
    SB1 = B.switch_map(r, W, st.mean, rm, st.Halo("out"))
    SC1 = B.switch_map(r, W, st.mean, st.Use(), st.Halo("in"))
    assert same(A1, B1, SA1, SB1)
    assert approx(A1, mat(g, "mean_remove_window1_5x6"))
    assert same(C1, SC1)
    assert same(A1[1:-1, 1:-1], C1, SC1, r[1:-1, 1:-1])
    A1 = B.map(r, W, st.sum, rm, st.Conditional())
    B1 = B.map(r, W, st.sum, rm, st.Halo("out"))
    C1 = B.map(r, W, st.sum, st.Use(), st.Halo("in"))
    SA1 = B.switch_map(r, W, st.sum, rm, st.Conditional())
    SB1 = B.switch_map(r, W, st.sum, rm, st.Halo("out"))
    SC1 = B.switch_map(r, W, st.sum, st.Use(), st.Halo("in"))
    assert same(A1, B1, SA1, SB1)
    assert same(A1[1:-1, 1:-1], C1, SC1, mat(g, "sum_use_halo_in_window1_5x6_interior"))


def case_wrap(B, st, g):
    """test/array.jl:164-209 (Wrap, 1-D and 2-D)."""
    x = np.arange(1.0, 6.0)
    s = st.Window(1, 1)
    A1 = B.map(x, s, st.mean, st.Wrap(), st.Conditional())
    B1 = B.map(x, s, st.mean, st.Wrap(), st.Halo("out"))
    C1 = B.map(x, s, st.mean, st.Wrap(), st.Halo("in"))
    SA1 = B.switch_map(x, s, st.mean, st.Wrap(), st.Conditional())
    SB1 = B.switch_map(x, s, st.mean, st.Wrap(), st.Halo("out"))
    SC1 = B.switch_map(x, s, st.mean, st.Wrap(), st.Halo("in"))
    assert same(A1, B1, SA1, np.array(g["mean_wrap_window1_1d"]["data"]))
    assert same(SB1, A1)
    assert same(C1, SC1, np.array(g["mean_wrap_halo_in_window1_1d"]["data"]))
    r = r_5x6()
    s = st.Window(1, 2)
    A1 = B.map(r, s, st.mean, st.Wrap(), st.Conditional())
    B1 = B.map(r, s, st.mean, st.Wrap(), st.Halo("out"))
    C1 = B.map(r, s, st.mean, st.Wrap(), st.Halo("in"))
    SA1 = B.switch_map(r, s, st.mean, st.Wrap(), st.Conditional())
    SB1 = B.switch_map(r, s, st.mean, st.Wrap(), st.Halo("out"))
    SC1 = B.switch_map(r, s, st.mean, st.Wrap(), st.Halo("in"))
    assert same(A1, B1, SA1, SB1)
    assert approx(A1, mat(g, "mean_wrap_window1_5x6"))
    assert same(C1, SC1)


def case_reflect(B, st, g):
    """test/array.jl:211-260 (Reflect, 1-D and 2-D)."""
    x = np.arange(1.0, 6.0)
    s = st.Window(1, 1)
    A1 = B.map(x, s, st.mean, st.Reflect(), st.Conditional())
    B1 = B.map(x, s, st.mean, st.Reflect(), st.Halo("out"))
    C1 = B.map(x, s, st.mean, st.Reflect(), st.Halo("in"))
    SA1 = B.switch_map(x, s, st.mean, st.Reflect(), st.Conditional())
    SB1 = B.switch_map(x, s, st.mean, st.Reflect(), st.Halo("out"))
    SC1 = B.switch_map(x, s, st.mean, st.Reflect(), st.Halo("in"))
    assert same(A1, B1, SA1, SB1)
    assert approx(A1, g["mean_reflect_window1_1d"]["data"])
    assert same(C1, SC1)
    assert approx(C1, g["mean_reflect_halo_in_window1_1d"]["data"])
    r = r_5x6()
    s = st.Window(1, 2)
    A1 = B.map(r, s, st.mean, st.Reflect(), st.Conditional())
    B1 = B.map(r, s, st.mean, st.Reflect(), st.Halo("out"))
    C1 = B.map(r, s, st.mean, st.Reflect(), st.Halo("in"))
    SA1 = B.switch_map(r, s, st.mean, st.Reflect(), st.Conditional())
    SB1 = B.switch_map(r, s, st.mean, st.Reflect(), st.Halo("out"))
    SC1 = B.switch_map(r, s, st.mean, st.Reflect(), st.Halo("in"))
    assert same(A1, B1, SA1, SB1)
    assert approx(A1, mat(g, "mean_reflect_window1_5x6"))
    assert same(C1, SC1)
    assert same(A1[2:-2, 2:-2], C1[1:-1, 1:-1], SC1[1:-1, 1:-1])
    assert same(A1[1:-1, 1:-1], B1[1:-1, 1:-1], SA1[1:-1, 1:-1], SB1[1:-1, 1:-1], r[1:-1, 1:-1])
    assert not same(A1[1:-1, 1:-1], C1)


def case_window_line_equivalence(B, st, g, rng):
    """test/array.jl:81-86 and :109-118: a lower-dimensional window equals the line stencil."""
    r = np.asfortranarray(rng.random((40, 30)))
    a = B.map(r, st.Vertical(1, 2), st.sum, st.Remove(0.0), st.Conditional())
    b = B.map(r, st.Window(1, 1), st.sum, st.Remove(0.0), st.Conditional())
    assert same(a, b)
    r3 = np.asfortranarray(rng.random((12, 11, 10)))
    pos3 = st.Positional((-1, -1, 0), (0, -1, 0), (1, -1, 0), (-1, 0, 0), (0, 0, 0), (1, 0, 0),
                         (-1, 1, 0), (0, 1, 0), (1, 1, 0))
    a = B.map(r3, st.Window(1, 2), st.sum, st.Remove(0.0), st.Conditional())
    b = B.map(r3, pos3, st.sum, st.Remove(0.0), st.Conditional())
    assert same(a, b)


def _onehot_neighbors(B, st, arr, stencil, I, boundary=None):
    """neighbors(StencilArray(arr, stencil), I) through the map kernel: kernelproduct with a
    one-hot weight vector picks neighbour k exactly (0 + v*1, other terms absent)."""
    boundary = st.Remove(0) if boundary is None else boundary
    vals = []
    L = len(stencil)
    idx = tuple(i - 1 for i in I)
    for k in range(L):
        w = np.zeros(L)
        w[k] = 1.0
        kern = st.Kernel(stencil, w)
        out = B.map(arr, kern, st.kernelproduct, boundary, st.Conditional())
        vals.append(out[idx])
    return vals


def case_neighbor_goldens(B, st, g):
    """Neighbour values of the shape tests (test/stencils.jl:59-184)."""
    init = mat(g, "init_6x6").astype(np.int64)
    win = mat(g, "win_5x5").astype(np.int64)
    for shape, name in ((st.VonNeumann(1), "neighbors_vonneumann_init_at_2_2"),
                        (st.Annulus(1), "neighbors_annulus_init_at_2_2"),
                        (st.Ordinal(1), "neighbors_ordinal_init_at_2_2"),
                        (st.Cardinal(1), "neighbors_cardinal_init_at_2_2")):
        got = _onehot_neighbors(B, st, np.asfortranarray(init), shape, (2, 2))
        assert got == g[name]["data"], name
    h1 = st.Positional(*[tuple(o) for o in g["positional_h1_offsets"]["data"]])
    assert _onehot_neighbors(B, st, np.asfortranarray(win), h1, (3, 3)) == g["neighbors_positional_h1_win_at_3_3"]["data"]
    h2 = st.Positional(*[tuple(o) for o in g["positional_h2_offsets"]["data"]])
    assert _onehot_neighbors(B, st, np.asfortranarray(win), h2, (3, 3)) == g["neighbors_positional_h2_win_at_3_3"]["data"]
    A5 = np.asfortranarray(mat(g, "rectangle_A_5x5").astype(np.int64))
    r1 = st.Rectangle((-1, 0), (-2, 1))
    assert _onehot_neighbors(B, st, A5, r1, (3, 3)) == g["neighbors_rectangle_h1_at_3_3"]["data"]
    A3 = np.asfortranarray(np.stack([A5, A5, A5], axis=2))
    r3 = st.Rectangle((-1, 0), (0, 1), (1, 1))
    assert _onehot_neighbors(B, st, A3, r3, (2, 2, 1)) == g["neighbors_rectangle_h3_3d_at_2_2_1"]["data"]


def case_kernelproduct_goldens(B, st, g):
    """test/stencils.jl:268-304: kernelproduct on the 3x3 array reshape(1:9, 3, 3) at its centre."""
    a = np.asfortranarray(np.arange(1, 10, dtype=np.int64).reshape(3, 3, order="F"))
    out = B.map(a, st.Kernel(st.Window(1), np.arange(1.0, 10.0)), st.kernelproduct, st.Remove(0),
                st.Conditional())
    assert out[1, 1] == sum(i * i for i in range(1, 10))
    vals = [1.0, 2, 3, 4, 6, 7, 8, 9]
    out = B.map(a, st.Kernel(st.Moore(1), vals), st.kernelproduct, st.Remove(0), st.Conditional())
    assert out[1, 1] == sum(v * v for v in vals)
    off = [tuple(o) for o in g["kernel_positional_offsets"]["data"]]
    out = B.map(a, st.Kernel(st.Positional(*off), [1.0, 2, 3, 4]), st.kernelproduct, st.Remove(0),
                st.Conditional())
    assert out[1, 1] == 60


def case_named_goldens(B, st, g):
    """test/stencils.jl:205-239: sums of named neighbours, as kernelproducts over sub-tables."""
    win = np.asfortranarray(mat(g, "win_5x5").astype(np.int64))
    # s.n + s.w + center(s), names n=(-1,0), e=(0,-1), w=(1,0), s=(0,1)
    k = st.Kernel(st.Positional((-1, 0), (1, 0), (0, 0)), [1.0, 1.0, 1.0])
    out = B.map(win, k, st.kernelproduct, st.Remove(0), st.Conditional())
    assert np.array_equal(out, mat(g, "named_n_w_center_minus_win") + win)
    # Cardinal(1) names (E, S, N, W): s.W + s.S
    card = st.NamedStencil(st.Cardinal(1))
    o = dict(zip(card.names, card.offsets()))
    out = B.map(win, st.Kernel(st.Positional(o["W"], o["S"]), [1.0, 1.0]), st.kernelproduct, st.Remove(0),
                st.Conditional())
    assert np.array_equal(out, mat(g, "named_cardinal_W_plus_S"))
    # Ordinal(1) names (SE, NE, SW, NW): s.NE + s.NW
    ordn = st.NamedStencil(st.Ordinal(1))
    o = dict(zip(ordn.names, ordn.offsets()))
    out = B.map(win, st.Kernel(st.Positional(o["NE"], o["NW"]), [1.0, 1.0]), st.kernelproduct, st.Remove(0),
                st.Conditional())
    assert np.array_equal(out, mat(g, "named_ordinal_NE_plus_NW"))


ALL_CASES = [case_remove_use, case_wrap, case_reflect, case_neighbor_goldens, case_kernelproduct_goldens,
             case_named_goldens]
