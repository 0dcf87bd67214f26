"""stc_life_steps_noalloc: the Life path for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc: code running inside a stream capture or a caller-managed
memory pool, or a host runtime that must stay the only owner of device memory.  This entry point
keeps its packed scratch in a fixed array inside the library instead of allocating it.  The test
calls it through the C ABI twice in a row and checks each result, bit for bit, against the
allocating entry point stc_map_steps on the same input.  (Life is integer work: exact equality is
the tolerance every other Life test uses.)  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, abi, st, fn, a_dev, b_dev, bnd, pad, steps):
    stl = abi.LoweredStencil(st.Moore(1))
    op = abi.lower_op(st.life)
    padi = st.Halo("in") if isinstance(pad, st.Halo) else st.Conditional()
    bc = abi.lower_bc(bnd, padi)
    ga, gb = abi.grid_from_torch(a_dev), abi.grid_from_torch(b_dev)
    out = C.c_int32(-1)
    if fn == "noalloc":
        rc = lib.stc_life_steps_noalloc(C.byref(ga), C.byref(gb), C.byref(stl.desc), C.byref(op), C.byref(bc), steps,
                                        C.byref(out), None)
    else:
        rc = lib.stc_map_steps(C.byref(ga), C.byref(gb), C.byref(stl.desc), C.byref(op), C.byref(bc), steps,
                               C.byref(out), None, 0)
    return rc, out.value


def _parents(st, a, pad):
    dev = st.to_device(a)
    S = st.SwitchingStencilArray(dev, st.Moore(1), st.Wrap(), pad)
    return S.source, S.dest


def test_noalloc_matches_allocating_path_twice(cuda, lib, st, abi):
    import torch
    rng = np.random.default_rng(2024)
    cases = [((4096, 4096), st.Wrap(), st.Halo("out"), 100),
             ((1024, 700), st.Remove(0), st.Conditional(), 37)]
    for shape, bnd, pad, steps in cases:            # two calls in a row, different grids
        a = np.asfortranarray((rng.random(shape) < 0.3).astype(np.uint8))
        na, nb = _parents(st, a, pad)
        ra, rb = _parents(st, a, pad)
        rc1, in_b1 = _run(lib, abi, st, "noalloc", na, nb, bnd, pad, steps)
        rc2, in_b2 = _run(lib, abi, st, "alloc", ra, rb, bnd, pad, steps)
        torch.cuda.synchronize()
        assert rc1 == 0 and rc2 == 0, (rc1, rc2)
        assert in_b1 == in_b2
        got = (nb if in_b1 else na).cpu().numpy()
        want = (rb if in_b2 else ra).cpu().numpy()
        if isinstance(pad, st.Halo):
            got, want = got[1:-1, 1:-1], want[1:-1, 1:-1]
        assert np.array_equal(got, want)
        prev_got = (na if in_b1 else nb).cpu().numpy()
        prev_want = (ra if in_b2 else rb).cpu().numpy()
        if isinstance(pad, st.Halo):
            prev_got, prev_want = prev_got[1:-1, 1:-1], prev_want[1:-1, 1:-1]
        assert np.array_equal(prev_got, prev_want)


def test_noalloc_rejects_grids_beyond_its_scratch(cuda, lib, st, abi):
    import torch
    a = st.colmajor_zeros((8192, 4096), torch.uint8)
    b = st.colmajor_zeros((8192, 4096), torch.uint8)
    rc, _ = _run(lib, abi, st, "noalloc", a, b, st.Wrap(), st.Conditional(), 3)
    assert rc == -12   # STC_ERR_TOO_LARGE
    odd = st.colmajor_zeros((100, 64), torch.uint8)
    odd2 = st.colmajor_zeros((100, 64), torch.uint8)
    rc, _ = _run(lib, abi, st, "noalloc", odd, odd2, st.Wrap(), st.Conditional(), 3)
    assert rc == -4    # width not a multiple of 32: not this path
