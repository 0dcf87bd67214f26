"""stc_life_steps_noalloc: the Life path for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc: a host whose device memory is all handed out by its own pool
or caching allocator (CUDA.jl's pool, a framework's allocator, an embedded host that reserved the
whole device), so that an allocation by the library would fail or take memory promised elsewhere.
This entry point keeps its packed scratch in a fixed array inside the library instead of
allocating it.  The tests call it through the C ABI, two calls in a row on different grids, and
check each result, bit for bit, against the allocating entry point stc_map_steps on the same
input.  (Life is integer work: exact equality is the tolerance every other Life test uses.)  This
file is collected last on purpose.
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


def _parents(st, a, pad, tdtype):
    import torch
    dev = st.to_device(a).to(tdtype)
    S = st.SwitchingStencilArray(dev, st.Moore(1), st.Wrap(), pad)
    return S.source, S.dest


def _interior(t, pad, st):
    x = t.to(dtype=__import__("torch").int64).cpu().numpy()
    return x[1:-1, 1:-1] if isinstance(pad, st.Halo) else x


def _compare_pair(lib, abi, st, a, bnd, pad, steps, tdtype):
    import torch
    na, nb = _parents(st, a, pad, tdtype)
    ra, rb = _parents(st, a, pad, tdtype)
    rc1, in_b1 = _run(lib, abi, st, "noalloc", na, nb, bnd, pad, steps)
    rc2, in_b2 = _run(lib, abi, st, "alloc", ra, rb, bnd, pad, steps)
    torch.cuda.synchronize()
    assert rc1 == 0 and rc2 == 0, (rc1, rc2)
    assert in_b1 == in_b2
    assert np.array_equal(_interior(nb if in_b1 else na, pad, st), _interior(rb if in_b2 else ra, pad, st))
    if steps > 0:   # the other parent holds generation steps - 1 in both paths
        assert np.array_equal(_interior(na if in_b1 else nb, pad, st), _interior(ra if in_b2 else rb, pad, st))


def test_noalloc_matches_allocating_path_twice(cuda, lib, st, abi):
    import torch
    rng = np.random.default_rng(2024)
    cases = [((4096, 4096), st.Wrap(), st.Halo("out"), 100),
             ((1024, 700), st.Remove(0), st.Conditional(), 37),
             ((1001, 300), st.Wrap(), st.Conditional(), 29)]      # rows with spare bits
    for shape, bnd, pad, steps in cases:            # two calls in a row, different grids
        a = np.asfortranarray((rng.random(shape) < 0.3).astype(np.uint8))
        _compare_pair(lib, abi, st, a, bnd, pad, steps, torch.uint8)


@pytest.mark.parametrize("dtype", ["bool", "i32", "i64"])
@pytest.mark.parametrize("steps", [0, 1, 2, 19])
def test_noalloc_dtypes_and_step_counts(cuda, lib, st, abi, dtype, steps):
    import torch
    tdt = {"bool": torch.bool, "i32": torch.int32, "i64": torch.int64}[dtype]
    rng = np.random.default_rng(7 + steps)
    for shape, bnd, pad in (((256, 130), st.Wrap(), st.Conditional()), ((96, 75), st.Remove(0), st.Halo("out"))):
        a = np.asfortranarray((rng.random(shape) < 0.3).astype(np.uint8))
        _compare_pair(lib, abi, st, a, bnd, pad, steps, tdt)


def test_noalloc_widest_rows(cuda, lib, st, abi):
    """Rows of 16384 cells (512 packed words, one per thread of the 512-thread CTA), the widest accepted."""
    import torch
    rng = np.random.default_rng(99)
    a = np.asfortranarray((rng.random((16384, 1024)) < 0.3).astype(np.uint8))
    _compare_pair(lib, abi, st, a, st.Wrap(), st.Conditional(), 21, torch.uint8)


def test_noalloc_rejects_grids_beyond_its_scratch(cuda, lib, st, abi):
    import torch
    a = st.colmajor_zeros((8192, 4096), torch.uint8)
    b = st.colmajor_zeros((8192, 4096), torch.uint8)
    rc, _ = _run(lib, abi, st, "noalloc", a, b, st.Wrap(), st.Conditional(), 3)
    assert rc == -12   # STC_ERR_TOO_LARGE
    narrow = st.colmajor_zeros((20, 64), torch.uint8)
    narrow2 = st.colmajor_zeros((20, 64), torch.uint8)
    rc, _ = _run(lib, abi, st, "noalloc", narrow, narrow2, st.Wrap(), st.Conditional(), 3)
    assert rc == -4    # rows shorter than 32 cells: not this path
    # 32768 x 512 holds exactly 4096^2 cells but its rows (1024 words) are wider than the CTA
    wide = st.colmajor_zeros((32768, 512), torch.uint8)
    wide2 = st.colmajor_zeros((32768, 512), torch.uint8)
    rc, _ = _run(lib, abi, st, "noalloc", wide, wide2, st.Wrap(), st.Conditional(), 3)
    assert rc == -4    # STC_ERR_UNSUPPORTED
