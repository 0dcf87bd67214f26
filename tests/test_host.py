"""Host-side logic of the reference API mirror: sizes per padding mode, argument errors, indices."""
import numpy as np
import pytest


def test_sizes_1d_2d_3d(st):
    """test/array.jl:16-107: parent and logical sizes across Conditional / Halo(:out) / Halo(:in)."""
    r = np.random.default_rng(0).random(100)
    A = st.StencilArray(r, st.VonNeumann(3, 1), st.Remove(0.0), st.Conditional())
    B = st.StencilArray(r, st.Window(10, 1), st.Remove(0.0), st.Halo("out"))
    C = st.StencilArray(r, st.Moore(10, 1), st.Remove(0.0), st.Halo("in"))
    sA = st.SwitchingStencilArray(r, st.Window(10, 1), st.Remove(0.0), st.Conditional())
    sB = st.SwitchingStencilArray(r, st.Window(10, 1), st.Remove(0.0), st.Halo("out"))
    sC = st.SwitchingStencilArray(r.copy(), st.Window(10, 1), st.Remove(0.0), st.Halo("in"))
    assert sA.source is not sA.dest
    assert A.shape == A.parent.shape == sA.shape == (100,)
    assert B.shape == sB.shape == (100,)
    assert B.parent.shape == sB.parent.shape == (120,)
    assert C.shape == sC.shape == (80,)
    assert C.parent.shape == sC.parent.shape == (100,)
    r2 = np.random.default_rng(1).random((100, 100))
    assert st.StencilArray(r2, st.Window(10), st.Remove(0.0), st.Halo("out")).parent.shape == (120, 120)
    assert st.StencilArray(r2, st.Moore(10), st.Remove(0.0), st.Halo("in")).shape == (80, 80)
    r3 = np.zeros((30, 30, 30))
    assert st.StencilArray(r3, st.Moore(10, 3), st.Remove(0.0), st.Halo("out")).parent.shape == (50, 50, 50)
    assert st.StencilArray(r3, st.VonNeumann(10, 3), st.Remove(0.0), st.Halo("in")).shape == (10, 10, 10)


def test_halo_out_copies_interior(st):
    a = np.asfortranarray(np.arange(12.0).reshape(3, 4, order="F"))
    B = st.StencilArray(a, st.Moore(1), st.Wrap(), st.Halo("out"))
    assert np.array_equal(B.array(), a)


def test_radius_check(st):
    """StencilArray requires radius < each axis (src/array.jl:451-453)."""
    with pytest.raises(st.ArgumentError):
        st.StencilArray(np.zeros((3, 10)), st.Window(3))
    with pytest.raises(st.ArgumentError):
        st.SwitchingStencilArray(np.zeros(4), st.Window(4, 1))
    st.StencilArray(np.zeros((3, 10)), st.Window(3), padding=st.Halo("out"))  # padded parent is large enough


def test_switching_size_mismatch(st):
    with pytest.raises(st.ArgumentError):
        st.SwitchingStencilArray(np.zeros((5, 5)), st.Moore(1), st.Wrap(), st.Conditional(), _dest=np.zeros((5, 6)))


def test_indices_goldens(st, goldens):
    """test/array.jl:5-14: indices under Remove, Wrap, Reflect (1-based, as the reference)."""
    z = np.zeros((4, 4))
    t = lambda n: tuple(tuple(o) for o in goldens[n]["data"])
    A = st.StencilArray(z, st.Moore(1), st.Remove(0.0), st.Conditional())
    assert A.indices((1, 1)) == t("indices_remove_moore_4x4_at_1_1")
    A = st.StencilArray(z, st.Moore(1), st.Wrap(), st.Conditional())
    assert A.indices((1, 1)) == t("indices_wrap_moore_4x4_at_1_1")
    A = st.StencilArray(z, st.Moore(1), st.Reflect(), st.Conditional())
    assert A.indices((1, 1)) == t("indices_reflect_moore_4x4_at_1_1")
    S = st.SwitchingStencilArray(z, st.Moore(1), st.Reflect(), st.Conditional())
    assert S.indices((1, 1)) == t("indices_switching_reflect_moore_4x4_at_1_1")


def test_host_neighbors_goldens(st, goldens):
    """neighbors(A, I) on host parents (test/stencils.jl:62-70, :145-146)."""
    init = np.asfortranarray(np.array(goldens["init_6x6"]["data"], dtype=np.int64))
    A = st.StencilArray(init, st.VonNeumann(1))
    assert A.neighbors((2, 2)) == goldens["neighbors_vonneumann_init_at_2_2"]["data"]
    win = np.asfortranarray(np.array(goldens["win_5x5"]["data"], dtype=np.int64))
    h1 = st.Positional(*[tuple(o) for o in goldens["positional_h1_offsets"]["data"]])
    assert st.StencilArray(win, h1).neighbors((3, 3)) == goldens["neighbors_positional_h1_win_at_3_3"]["data"]


def test_unregistered_function(st):
    with pytest.raises(NotImplementedError):
        st.mapstencil(lambda h: 0, st.StencilArray(np.zeros((4, 4)), st.Moore(1)))


def test_remove_nothing_rejected(st, abi):
    with pytest.raises(ValueError):
        abi.lower_bc(st.Remove(), st.Conditional())


def test_result_dtypes(st, orc, abi):
    """Base._return_type of each registered reduction (src/gatherstencil.jl:41-56)."""
    assert orc.result_dtype(st.mean, abi.F64) == abi.F64
    assert orc.result_dtype(st.mean, abi.U8) == abi.F64
    assert orc.result_dtype(st.sum, abi.BOOL) == abi.I64
    assert orc.result_dtype(st.sum, abi.U8) == abi.U8
    assert orc.result_dtype(st.kernelproduct, abi.F32, abi.F32) == abi.F32
    assert orc.result_dtype(st.kernelproduct, abi.F32, abi.F64) == abi.F64
    assert orc.result_dtype(st.life, abi.U8) == abi.U8
    with pytest.raises(NotImplementedError):
        orc.result_dtype(st.life, abi.F32)


def test_halo_out_parents_align_interior_rows(st):
    """pad_array for Halo{:out} on a torch parent: the reference's shape and contents, with the interior's
    rows starting on 128-byte lines (axis-1 stride a multiple of 128 bytes)."""
    import torch
    from stencils_gb300.array import halo_parent_zeros, pad_array
    for dt in (torch.float32, torch.float64, torch.bfloat16, torch.uint8, torch.int64):
        for R in (1, 2, 3):
            for shape in ((9,), (7, 5), (13, 6, 4)):
                t = halo_parent_zeros(shape, R, dt, "cpu")
                es = t.element_size()
                assert tuple(t.shape) == shape and t.stride(0) == 1
                if len(shape) > 1:
                    assert (t.stride(1) * es) % 128 == 0
                assert ((t.storage_offset() + R) * es) % 128 == 0
                assert not t.any()
    a = torch.from_numpy(np.asfortranarray(np.arange(35, dtype=np.float32).reshape(7, 5)))
    p = pad_array(st.Halo("out"), st.Moore(2), a)
    assert tuple(p.shape) == (11, 9)
    assert np.array_equal(p[2:-2, 2:-2].numpy(), a.numpy()) and float(p.sum()) == float(a.sum())


def test_lowered_stencil_cache_follows_radius_and_shape(st):
    """The per-stencil lowering is reused for the same stencil and redone for a copy with another radius
    (an enclosing Layered stencil's), so the descriptor always carries the stencil's own radius and shape."""
    from stencils_gb300 import _abi as A
    from stencils_gb300.stencil import with_radius
    s = st.Window(1)
    a = A.lowered_stencil(s)
    assert A.lowered_stencil(s) is a
    assert (a.desc.radius, a.desc.shape) == (1, s.shape_id)
    w = with_radius(s, 3)
    b = A.lowered_stencil(w)
    assert b is not a and (b.desc.radius, b.desc.shape) == (3, w.shape_id)
    assert A.lowered_stencil(s).desc.radius == 1
    w.radius = 2   # changed in place: lowered again
    assert A.lowered_stencil(w).desc.radius == 2
    k = st.Kernel(st.Window(1), list(range(9)))
    assert A.lowered_stencil(k) is not A.lowered_stencil(k)   # kernels: weights may change, never reused
