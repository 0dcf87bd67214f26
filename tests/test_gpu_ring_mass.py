"""Direct checks of two library outputs that the maps only use indirectly.

* stc_update_boundary (update_boundary!, src/array.jl:195-233): the whole Halo parent after the call,
  ring slabs and corners included, equals the oracle's restatement bit for bit, for Remove / Wrap /
  Reflect, 1D-3D, radius 1-3.
* stc_mass: the FP64 compensated total equals the correctly rounded sum of the grid (math.fsum) to within
  two ulps, on uniform data and on data with a large common offset, where plain summation drifts.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("bname", ["remove", "wrap", "reflect"])
@pytest.mark.parametrize("shape,R", [((37,), 2), ((29, 17), 1), ((21, 14), 3), ((13, 11, 9), 1), ((12, 9, 10), 2)])
@pytest.mark.parametrize("code", ["f64", "f32", "u8"])
def test_update_boundary_ring_matches_oracle(cuda, st, orc, abi, bname, shape, R, code):
    rng = np.random.default_rng(sum(shape) * 7 + R)
    dt = {"f64": np.float64, "f32": np.float32, "u8": np.uint8}[code]
    padded = tuple(s + 2 * R for s in shape)
    parent = rng.random(padded) * 100
    parent = np.asfortranarray(parent.astype(dt))        # the ring starts as garbage
    bnd = {"remove": st.Remove(7 if code == "u8" else 0.5), "wrap": st.Wrap(), "reflect": st.Reflect()}[bname]
    hood = st.Window(R, len(shape)) if len(shape) <= 2 else st.Moore(R, 3)
    d = st.to_device(parent)
    S = st.StencilArray.from_parent(d, hood, bnd, st.Halo("in"))
    st.update_boundary_(S)
    got = st.to_host(d)
    want = parent.copy(order="F")
    orc.update_boundary(want, {"f64": abi.F64, "f32": abi.F32, "u8": abi.U8}[code], R, bnd, st.Halo("in"))
    assert got.tobytes(order="F") == want.tobytes(order="F")


def _ulp(x: float) -> float:
    return math.ulp(x) if x != 0 else math.ulp(0.0)


def test_mass_matches_exact_sum(cuda, st):
    rng = np.random.default_rng(12)
    a = np.asfortranarray(rng.random((4096, 4096), dtype=np.float32))
    exact = math.fsum(a.astype(np.float64).ravel())
    got = st.mass(st.to_device(a))
    assert abs(got - exact) <= 2 * _ulp(exact), (got, exact)
    # a large common offset: every plain addition to a running total near 1e14 drops the low bits of
    # the uniform part (about 8 absolute after 1M terms); the compensated total keeps them
    b = np.asfortranarray(1e8 + rng.random((1024, 1024)))
    exact = math.fsum(b.ravel())
    got = st.mass(st.to_device(b))
    assert abs(got - exact) <= 2 * _ulp(exact), (got, exact)
    # a Halo parent: only the logical interior counts
    c = np.asfortranarray(rng.random((66, 50)))
    c_in = c[2:-2, 2:-2]
    got = st.mass(st.to_device(c), radius=2, padding=st.Halo("in"))
    exact = math.fsum(c_in.ravel())
    assert abs(got - exact) <= 2 * _ulp(exact)
