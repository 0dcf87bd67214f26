"""Offset tables of every shape against the reference's own test expectations (test/stencils.jl)."""
import math

import pytest


def offs(g, name):
    return tuple(tuple(o) for o in g[name]["data"])


def test_moore(st, goldens):
    m = st.Moore(1)
    assert m.offsets() == offs(goldens, "offsets_moore_1_2")
    assert m.radius == 1 and m.diameter() == 3 and len(m) == 8
    sq2 = math.sqrt(2)
    assert m.distances() == (sq2, 1.0, sq2, 1.0, 1.0, sq2, 1.0, sq2)   # test/stencils.jl:32
    assert m.indices((1, 1)) == ((0, 0), (1, 0), (2, 0), (0, 1), (2, 1), (0, 2), (1, 2), (2, 2))  # :29-30


def test_window(st, goldens):
    w = st.Window(1)
    assert w.offsets() == offs(goldens, "offsets_window_1_2")
    assert st.Window(1) == st.Window(1, 2)   # test/stencils.jl:37
    assert len(w) == 9
    # 1-D windows keep the first component of the reference's 2-tuples
    assert st.Window(2, 1).offsets() == ((-2,), (-1,), (0,), (1,), (2,))
    with pytest.raises(ValueError):
        st.Window(1, 3)


def test_vonneumann(st, goldens):
    assert st.VonNeumann(1).offsets() == offs(goldens, "offsets_vonneumann_1_2")
    assert st.VonNeumann(2).offsets() == offs(goldens, "offsets_vonneumann_2_2")
    assert len(st.VonNeumann(1, 3)) == 6


def test_annulus_ordinal_cardinal(st, goldens):
    assert st.Annulus(1).offsets() == offs(goldens, "offsets_annulus_1")
    assert st.Annulus(2).offsets() == offs(goldens, "offsets_annulus_2")
    assert st.Ordinal(1).offsets() == offs(goldens, "offsets_ordinal_1")
    assert st.Ordinal(2).offsets() == offs(goldens, "offsets_ordinal_2")
    assert st.Cardinal(1).offsets() == offs(goldens, "offsets_cardinal_1")
    assert st.Cardinal(2).offsets() == offs(goldens, "offsets_cardinal_2")


def test_positional_radius_quirk(st, goldens):
    h1 = st.Positional(*offs(goldens, "positional_h1_offsets"))
    assert h1.radius == 2 and len(h1) == 5          # test/stencils.jl:143-144
    h2 = st.Positional(*offs(goldens, "positional_h2_offsets"))
    assert h2.radius == 1 and len(h2) == 4          # :151-152
    # radius is maximum(map(maximum, O)), not the largest absolute offset
    q = st.Positional((-2, -2), (-1, -1))
    assert q.radius == -1 and q.max_abs_offset() == 2


def test_rectangle(st):
    h1 = st.Rectangle((-1, 0), (-2, 1))
    assert h1.radius == 2 and len(h1) == 8          # test/stencils.jl:167-168
    h3 = st.Rectangle((-1, 0), (0, 1), (1, 1))
    assert h3.radius == 1 and len(h3) == 4          # :178-179


def test_circle_cross_counts(st):
    assert len(st.Circle(3)) == 37
    assert len(st.Cross(2)) == 9
    assert len(st.Window(3)) == 49
    assert st.Circle(1).offsets() == st.Window(1).offsets()
    for sh in (st.Window(2), st.Moore(1, 3), st.VonNeumann(1, 3), st.Circle(3), st.Cross(2, 3)):
        assert sh.is_sorted_colmajor()


def test_named(st):
    ns = st.NamedStencil(n=(-1, 0), e=(0, -1), w=(1, 0), s=(0, 1))
    assert ns.radius == 1 and len(ns) == 4
    # NamedStencil{(:n,:e,:w,:s)}(VonNeumann()) names VonNeumann's offsets in order (test/stencils.jl:215;
    # the reference's `==` there compares the two empty neighbour vectors, not the offsets)
    nv = st.NamedStencil(st.VonNeumann(1), names=("n", "e", "w", "s"))
    assert dict(zip(nv.names, nv.offsets()))["n"] == (0, -1)
    with pytest.raises(ValueError):
        st.NamedStencil(st.VonNeumann(1), names=("n", "s"))                    # :216
    assert st.NamedStencil(st.Cardinal(1)).names == ("E", "S", "N", "W")


def test_kernel(st):
    import numpy as np
    k = st.Kernel(st.Window(1), np.arange(1, 10).reshape(3, 3, order="F"))
    assert k.weights == tuple(float(i) for i in range(1, 10))
    with pytest.raises(ValueError):
        st.Kernel(st.Window(2), list(range(9)))       # test/stencils.jl:272
    g = st.Kernel(lambda d: math.exp(-d * d / 2), st.Window(1))
    assert len(g.weights) == 9 and g.weights[4] == 1.0
    assert st.Kernel(np.ones((3, 3))).stencil == st.Window(1)
