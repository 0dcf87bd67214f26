"""Temporally blocked 2D multi-step maps (K7, Float32): both final states bit-exact against the oracle's
per-step gather, and the blocked kernel is the one that ran."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_gpu(st, a, stencil, red, bnd, pad, steps):
    from stencils_gb300 import _lib
    S = st.SwitchingStencilArray(st.to_device(a), stencil, bnd, pad)
    first = S.source.data_ptr()
    _lib.profile_enable(True)
    try:
        S = st.mapstencil_(red, S, steps=steps)
        kern = _lib.profile_report()
    finally:
        _lib.profile_enable(False)
    # state n in the parent the reference's loop leaves it in: the first one after an even number of steps
    assert (S.source.data_ptr() == first) == (steps % 2 == 0)
    res, prev = S.source.cpu().numpy(), S.dest.cpu().numpy()
    if isinstance(pad, st.Halo):
        res, prev = res[1:-1, 1:-1], prev[1:-1, 1:-1]
    return np.asfortranarray(res), np.asfortranarray(prev), kern


def _run_oracle(st, orc, abi, a, stencil, red, bnd, steps):
    pa, pb = np.asfortranarray(a).copy(order="F"), np.asfortranarray(a).copy(order="F")
    in_b = orc.map_steps(pa, pb, abi.F32, stencil, red, bnd, st.Conditional(), steps, nthreads=orc.max_threads())
    return (pb, pa) if in_b else (pa, pb)


CASES = {
    "window_mean": lambda st: (st.Window(1), st.mean),
    "window_sum": lambda st: (st.Window(1), st.sum),
    "moore_mean": lambda st: (st.Moore(1), st.mean),
    "moore_sum": lambda st: (st.Moore(1), st.sum),
    "vn_mean": lambda st: (st.VonNeumann(1), st.mean),
    "vn_diffuse": lambda st: (st.VonNeumann(1), st.Diffusion(0.1)),
    "vn_sum": lambda st: (st.VonNeumann(1), st.sum),
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("bname", ["wrap", "remove0", "remove_q"])
@pytest.mark.parametrize("size,steps,levels", [((300, 170), 17, 8), ((50, 41), 26, 8), ((1031, 263), 21, 8),
                                               ((200, 90), 30, 8), ((300, 170), 9, 4), ((1031, 263), 14, 4)])
def test_blocked_2d_matches_oracle(cuda, st, orc, abi, monkeypatch, case, bname, size, steps, levels):
    """Grids smaller than one box, ragged in both axes, and several tiles wide; per-step maps after
    the blocked passes (two or more passes, then 1 to 8 steps); Wrap, Remove(0) and Remove(0.25)."""
    monkeypatch.setenv("STC_TB2_K", str(levels))
    rng = np.random.default_rng(steps * 131 + size[0] + len(bname) + len(case))
    a = np.asfortranarray(rng.random(size).astype(np.float32))
    stencil, red = CASES[case](st)
    bnd = {"wrap": st.Wrap(), "remove0": st.Remove(0.0), "remove_q": st.Remove(0.25)}[bname]
    got, gprev, kern = _run_gpu(st, a, stencil, red, bnd, st.Conditional(), steps)
    assert "tblock2d" in kern, kern
    want, wprev = _run_oracle(st, orc, abi, a, stencil, red, bnd, steps)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(gprev.view(np.uint32), wprev.view(np.uint32))   # state n-1 where the reference leaves it


@pytest.mark.parametrize("bname", ["wrap", "remove_q"])
def test_blocked_2d_halo_parents(cuda, st, orc, abi, bname):
    """Halo-padded parents: the blocked passes read and write the interiors; the tail steps refresh the ring."""
    rng = np.random.default_rng(7)
    a = np.asfortranarray(rng.random((257, 190)).astype(np.float32))
    bnd = {"wrap": st.Wrap(), "remove_q": st.Remove(0.25)}[bname]
    got, gprev, kern = _run_gpu(st, a, st.Window(1), st.mean, bnd, st.Halo("out"), 18)
    assert "tblock2d" in kern, kern
    want, wprev = _run_oracle(st, orc, abi, a, st.Window(1), st.mean, bnd, 18)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(gprev.view(np.uint32), wprev.view(np.uint32))


def test_blocked_2d_not_taken(cuda, st, orc, abi):
    """Reflect, Float64 and short runs keep the per-step path (and stay exact)."""
    rng = np.random.default_rng(9)
    a = np.asfortranarray(rng.random((140, 90)).astype(np.float32))
    got, _, kern = _run_gpu(st, a, st.Window(1), st.mean, st.Reflect(), st.Conditional(), 9)
    assert "tblock2d" not in kern
    want, _ = _run_oracle(st, orc, abi, a, st.Window(1), st.mean, st.Reflect(), 9)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    got, _, kern = _run_gpu(st, a, st.Window(1), st.mean, st.Wrap(), st.Conditional(), 16)
    assert "tblock2d" not in kern   # one pass of 8 would leave state n in the wrong parent: per-step


@pytest.mark.parametrize("kind", ["signed", "tiny", "huge", "zeros_and_tiny"])
def test_blocked_2d_mean_outside_the_fast_quotient_range(cuda, st, orc, abi, kind):
    """Tiles whose values leave [2^-64, 2^124] (or are negative) take the range-tested quotient; mixed
    grids take both kinds of tile in one pass.  Bit-exact either way."""
    rng = np.random.default_rng(len(kind))
    shape = (300, 170)
    a = rng.standard_normal(shape).astype(np.float32)
    if kind == "tiny":
        a = (np.abs(a) * 1e-30).astype(np.float32)
    elif kind == "huge":
        a = (np.abs(a) * 3e37).astype(np.float32)
    elif kind == "zeros_and_tiny":
        a = np.where(rng.random(shape) < 0.5, 0.0, np.abs(a)).astype(np.float32)
        a[:150, :] *= np.float32(1e-25)
    a = np.asfortranarray(a)
    got, gprev, kern = _run_gpu(st, a, st.Window(1), st.mean, st.Wrap(), st.Conditional(), 17)
    assert "tblock2d" in kern
    want, wprev = _run_oracle(st, orc, abi, a, st.Window(1), st.mean, st.Wrap(), 17)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(gprev.view(np.uint32), wprev.view(np.uint32))
