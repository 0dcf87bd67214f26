"""Pin the oracle: it must reproduce every golden vector of the reference's own tests for the
mapstencil path (test/array.jl, test/stencils.jl), read from tests/golden/reference_goldens.json."""
import numpy as np
import pytest

import _golden_cases as G
from _backends import OracleBackend


@pytest.fixture(scope="module")
def B(st, orc, abi):
    return OracleBackend(st, orc, abi)


@pytest.mark.parametrize("case", G.ALL_CASES, ids=lambda c: c.__name__)
def test_reference_goldens(case, B, st, goldens):
    case(B, st, goldens)


def test_window_line_equivalence(B, st, goldens):
    G.case_window_line_equivalence(B, st, goldens, np.random.default_rng(0))


def test_halo_fill_matches_reference_rules(st, orc, abi):
    """update_boundary! (src/array.jl:202-239) on a 4x5 interior with R=1, Wrap and Reflect."""
    a = np.asfortranarray(np.arange(1.0, 21.0).reshape(4, 5, order="F"))
    p = np.zeros((6, 7), order="F")
    p[1:5, 1:6] = a
    orc.update_boundary(p, abi.F64, 1, st.Wrap(), st.Halo("out"))
    assert np.array_equal(p[0, 1:6], a[3, :]) and np.array_equal(p[5, 1:6], a[0, :])
    assert np.array_equal(p[1:5, 0], a[:, 4]) and np.array_equal(p[1:5, 6], a[:, 0])
    assert p[0, 0] == a[3, 4] and p[5, 6] == a[0, 0]
    orc.update_boundary(p, abi.F64, 1, st.Reflect(), st.Halo("out"))
    assert np.array_equal(p[0, 1:6], a[1, :]) and np.array_equal(p[5, 1:6], a[2, :])
    assert p[0, 0] == a[1, 1]
    orc.update_boundary(p, abi.F64, 1, st.Remove(-3.0), st.Halo("out"))
    assert (p[0, :] == -3).all() and (p[:, 6] == -3).all()
    assert np.array_equal(p[1:5, 1:6], a)


def test_oracle_life_glider(st, orc, abi):
    """B3/S23 on a wrapped 8x8 board: a glider moves one cell diagonally every 4 generations."""
    g = np.zeros((8, 8), dtype=np.uint8, order="F")
    for x, y in ((1, 0), (2, 1), (0, 2), (1, 2), (2, 2)):
        g[x, y] = 1
    a, b = g.copy(order="F"), g.copy(order="F")
    in_b = orc.map_steps(a, b, abi.U8, st.Moore(1), st.life, st.Wrap(), st.Conditional(), 4)
    res = b if in_b else a
    assert np.array_equal(res, np.roll(np.roll(g, 1, 0), 1, 1))


def test_oracle_threads_agree(st, orc, abi):
    rng = np.random.default_rng(3)
    a = np.asfortranarray(rng.random((64, 48)))
    one = orc.map(a, abi.F64, st.Circle(2), st.mean, st.Wrap(), st.Conditional(), nthreads=1)
    many = orc.map(a, abi.F64, st.Circle(2), st.mean, st.Wrap(), st.Conditional(), nthreads=4)
    assert np.array_equal(one, many)
