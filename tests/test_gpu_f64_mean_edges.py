"""The Float64 Window(1) mean (the vector kernel: a left fold of __dadd_rn, then the integer division by 9)
bit-exact against the oracle on values that reach the edges of IEEE addition and division — all binades,
subnormal sums that become normal, exact ties, exponent gaps past the significand, overflow to +inf, +inf
inputs, zeros, negative regions, -0.0 and NaN — under Remove(0), Wrap and a negative Remove padval."""
import numpy as np
import pytest

from _backends import GpuBackend, OracleBackend

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(cuda, st, abi):
    return GpuBackend(st, abi)


@pytest.fixture(scope="module")
def ora(st, orc, abi):
    return OracleBackend(st, orc, abi)


SHAPE = (300, 170)


def _values(kind, rng):
    n = SHAPE
    if kind == "binades":
        return rng.random(n) * np.exp2(rng.integers(-1074, 1020, size=n).astype(np.float64))
    if kind == "blocks":
        # 8x8 blocks sharing a scale: whole windows of similar magnitude, as in smooth data
        blk = np.exp2(rng.integers(-1070, 1015, size=(n[0] // 8 + 1, n[1] // 8 + 1)).astype(np.float64))
        return rng.random(n) * np.kron(blk, np.ones((8, 8)))[: n[0], : n[1]]
    if kind == "ties":
        # 53-bit integers times small powers of two: sums often sit exactly half-way between doubles
        k = rng.integers(2**52, 2**53, size=n).astype(np.float64)
        return k * np.exp2(rng.integers(-3, 3, size=n).astype(np.float64))
    if kind == "subnormal":
        return rng.integers(0, 2**53, size=n).astype(np.uint64).view(np.float64)
    if kind == "gaps":
        return rng.random(n) * np.exp2(-rng.integers(0, 70, size=n).astype(np.float64))
    if kind == "overflow":
        return np.finfo(np.float64).max * (0.05 + rng.random(n))
    if kind == "inf":
        a = rng.random(n)
        a[rng.random(n) < 0.01] = np.inf
        return a
    if kind == "zeros":
        a = rng.random(n)
        a[rng.random(n) < 0.3] = 0.0
        return a
    if kind == "negative_regions":
        a = rng.random(n)
        a[100:140, 50:60] *= -1.0
        return a
    if kind == "minus_zero":
        a = rng.random(n)
        a[rng.random(n) < 0.001] = -0.0
        return a
    if kind == "nan":
        a = rng.random(n)
        a[rng.random(n) < 0.0005] = np.nan
        return a
    raise ValueError(kind)


KINDS = ["binades", "blocks", "ties", "subnormal", "gaps", "overflow", "inf", "zeros", "negative_regions",
         "minus_zero", "nan"]


def _same(got, want):
    gn, wn = np.isnan(got), np.isnan(want)
    assert np.array_equal(gn, wn)
    assert np.array_equal(got[~gn].view(np.uint64), want[~wn].view(np.uint64))


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("bname", ["remove0", "wrap", "remove_neg"])
def test_float64_mean_edges_bit_exact(gpu, ora, st, kind, bname):
    rng = np.random.default_rng(len(kind) * 7 + len(bname))
    a = np.asfortranarray(_values(kind, rng))
    bnd = {"remove0": st.Remove(0.0), "wrap": st.Wrap(), "remove_neg": st.Remove(-0.5)}[bname]
    with np.errstate(over="ignore", invalid="ignore"):
        want = ora.map(a, st.Window(1), st.mean, bnd, st.Conditional())
    got = gpu.map(a, st.Window(1), st.mean, bnd, st.Conditional())
    _same(got, want)
