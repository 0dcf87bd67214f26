"""Conway's Life through SwitchingStencilArray: the bit-packed, temporally blocked kernel against the
oracle's per-cell gather, bit for bit."""
import numpy as np
import pytest

from _backends import GpuBackend

pytestmark = pytest.mark.gpu


def _oracle_steps(orc, abi, st, a, code, rule, bnd, pad, steps, nthreads=None):
    """Reference: `steps` generations; returns (result, previous state) logical arrays."""
    nthreads = nthreads or orc.max_threads()
    halo = isinstance(pad, st.Halo)
    if halo:
        pa = np.zeros((a.shape[0] + 2, a.shape[1] + 2), dtype=a.dtype, order="F")
        pa[1:-1, 1:-1] = a
        padi = st.Halo("in")
    else:
        pa = np.array(a, order="F")
        padi = st.Conditional()
    pb = pa.copy(order="F")
    in_b = orc.map_steps(pa, pb, code, st.Moore(1), rule, bnd, padi, steps, nthreads=nthreads)
    res, prev = (pb, pa) if in_b else (pa, pb)
    if halo:
        res, prev = res[1:-1, 1:-1], prev[1:-1, 1:-1]
    return np.asfortranarray(res), np.asfortranarray(prev), in_b


def _gpu_run(st, dev_a, rule, bnd, pad, steps):
    from stencils_gb300 import _lib
    S = st.SwitchingStencilArray(dev_a, st.Moore(1), bnd, pad)
    _lib.profile_enable(True)
    S2 = st.mapstencil_(rule, S, steps=steps)
    kernels = _lib.profile_report()
    _lib.profile_enable(False)
    return S2, kernels


def _logical(t, pad, st):
    x = t.cpu().numpy() if t.dtype != __import__("torch").bool else t.cpu().numpy().astype(np.uint8)
    x = np.asfortranarray(x)
    if isinstance(pad, st.Halo):
        x = x[1:-1, 1:-1]
    return x


def test_life_4096_every_100_steps(cuda, st, orc, abi):
    """The Life benchmark grid: 4096x4096 UInt8, density 0.3 from seed 2, Wrap, Halo padding, 1000 generations,
    compared with the oracle after every 100."""
    rng = np.random.Generator(np.random.PCG64(2))
    a = np.asfortranarray((rng.random((4096, 4096)) < 0.3).astype(np.uint8))
    pad = st.Halo("out")
    S = st.SwitchingStencilArray(st.to_device(a), st.Moore(1), st.Wrap(), pad)
    ref = a.copy(order="F")
    from stencils_gb300 import _lib
    for chunk in range(10):
        _lib.profile_enable(True)
        S = st.mapstencil_(st.life, S, steps=100)
        kern = _lib.profile_report()
        _lib.profile_enable(False)
        assert ("life_coop" in kern or "life_block" in kern) and "map_shape_ldg" not in kern
        ref, _, _ = _oracle_steps(orc, abi, st, ref, abi.U8, st.life, st.Wrap(), st.Conditional(), 100)
        got = _logical(S.source, pad, st)
        assert np.array_equal(got, ref), f"differs after {100 * (chunk + 1)} generations"


@pytest.mark.parametrize("dtype", ["u8", "bool", "i32", "i64"])
@pytest.mark.parametrize("bname", ["wrap", "remove0"])
@pytest.mark.parametrize("pname", ["cond", "halo_out"])
@pytest.mark.parametrize("steps", [1, 2, 37])
def test_life_variants(cuda, st, orc, abi, dtype, bname, pname, steps):
    import torch
    rng = np.random.default_rng(steps * 7 + len(dtype))
    shape = (256, 77)
    bits = rng.random(shape) < 0.35
    code = {"u8": abi.U8, "bool": abi.BOOL, "i32": abi.I32, "i64": abi.I64}[dtype]
    npdt = {"u8": np.uint8, "bool": np.uint8, "i32": np.int32, "i64": np.int64}[dtype]
    a = np.asfortranarray(bits.astype(npdt))
    bnd = st.Wrap() if bname == "wrap" else st.Remove(0)
    pad = st.Halo("out") if pname == "halo_out" else st.Conditional()
    dev = st.to_device(a.astype(np.bool_)) if dtype == "bool" else st.to_device(a)
    S2, kern = _gpu_run(st, dev, st.life, bnd, pad, steps)
    assert "life_coop" in kern or "life_block" in kern
    res, prev, in_b = _oracle_steps(orc, abi, st, a, code, st.life, bnd, st.Conditional(), steps)
    assert np.array_equal(_logical(S2.source, pad, st).astype(npdt), res)
    if steps > 1:
        assert np.array_equal(_logical(S2.dest, pad, st).astype(npdt), prev)


def test_life_other_rule_and_small_grids(cuda, st, orc, abi):
    """HighLife (B36/S23) and grids shorter than the temporal block."""
    rng = np.random.default_rng(9)
    highlife = st.LifeRule((3, 6), (2, 3))
    seeds = st.LifeRule((2,), ())
    for shape, rule in (((64, 5), st.life), ((32, 3), highlife), ((512, 300), highlife), ((96, 40), seeds)):
        a = np.asfortranarray((rng.random(shape) < 0.4).astype(np.uint8))
        for bnd in (st.Wrap(), st.Remove(0)):
            S2, kern = _gpu_run(st, st.to_device(a), rule, bnd, st.Conditional(), 45)
            assert "life_coop" in kern or "life_block" in kern
            res, _, _ = _oracle_steps(orc, abi, st, a, abi.U8, rule, bnd, st.Conditional(), 45)
            assert np.array_equal(_logical(S2.source, st.Conditional(), st), res), (shape, rule.name, bnd)


def test_life_fallback_shapes_still_exact(cuda, st, orc, abi):
    """Rows shorter than 32 cells, Reflect and nonzero Remove take the per-generation kernel."""
    rng = np.random.default_rng(4)
    for shape, bnd in (((20, 64), st.Wrap()), ((128, 64), st.Reflect()), ((128, 64), st.Remove(1))):
        a = np.asfortranarray((rng.random(shape) < 0.4).astype(np.uint8))
        S2, kern = _gpu_run(st, st.to_device(a), st.life, bnd, st.Conditional(), 9)
        assert "life_block" not in kern and "life_coop" not in kern
        res, _, _ = _oracle_steps(orc, abi, st, a, abi.U8, st.life, bnd, st.Conditional(), 9)
        assert np.array_equal(_logical(S2.source, st.Conditional(), st), res)


@pytest.mark.parametrize("depth", ["1", "2", "5", "8", "13", "multi-launch"])
@pytest.mark.parametrize("bname", ["wrap", "remove0"])
def test_life_persistent_depths(cuda, st, orc, abi, monkeypatch, depth, bname):
    """The persistent kernel at several ghost depths (super-step lengths, including depths that do not
    divide the step count) and the multi-launch kernel, on a grid split over many bands."""
    from stencils_gb300 import _lib
    if depth == "multi-launch":
        monkeypatch.setenv("STC_LIFE_COOP", "0")
    else:
        monkeypatch.setenv("STC_LIFE_K", depth)
    rng = np.random.default_rng(31 + len(depth))
    a = np.asfortranarray((rng.random((1024, 700)) < 0.33).astype(np.uint8))
    bnd = st.Wrap() if bname == "wrap" else st.Remove(0)
    for steps in (1, 2, 29):
        S2, kern = _gpu_run(st, st.to_device(a), st.life, bnd, st.Conditional(), steps)
        assert ("life_block" if depth == "multi-launch" else "life_coop") in kern, kern
        res, prev, _ = _oracle_steps(orc, abi, st, a, abi.U8, st.life, bnd, st.Conditional(), steps)
        assert np.array_equal(_logical(S2.source, st.Conditional(), st), res), (depth, steps)
        if steps > 1:
            assert np.array_equal(_logical(S2.dest, st.Conditional(), st), prev), (depth, steps)


@pytest.mark.parametrize("depth", ["1", "2", "5", "8", "13"])
@pytest.mark.parametrize("bname", ["wrap", "remove0"])
def test_life_warp_rows_persistent_depths(cuda, st, orc, abi, monkeypatch, depth, bname):
    """Rows of 4096 cells (the warp-row split, whose first generation per super-step is split around the
    neighbour exchange) over 300 rows: bands of 2 to 13 rows, so some have no row that needs no ghost row
    (depths 1 and 2) and Remove clips the first and last bands; both states bit-exact against the oracle."""
    monkeypatch.setenv("STC_LIFE_K", depth)
    rng = np.random.default_rng(97 + len(depth) + len(bname))
    a = np.asfortranarray((rng.random((4096, 300)) < 0.33).astype(np.uint8))
    bnd = st.Wrap() if bname == "wrap" else st.Remove(0)
    for steps in (1, 2, 29):
        S2, kern = _gpu_run(st, st.to_device(a), st.life, bnd, st.Conditional(), steps)
        assert "life_coop" in kern, kern
        res, prev, _ = _oracle_steps(orc, abi, st, a, abi.U8, st.life, bnd, st.Conditional(), steps)
        assert np.array_equal(_logical(S2.source, st.Conditional(), st), res), (depth, steps)
        if steps > 1:
            assert np.array_equal(_logical(S2.dest, st.Conditional(), st), prev), (depth, steps)


def test_queued_calls_equal_waiting_calls(cuda, st):
    """mapstencil_(..., sync=False) only skips the wait: three queued 100-generation calls give the state
    one waiting 300-generation call gives."""
    import torch
    rng = np.random.default_rng(12)
    g = np.asfortranarray((rng.random((256, 192)) < 0.3).astype(np.uint8))
    S1 = st.SwitchingStencilArray(st.to_device(g), st.Moore(1), st.Wrap(), st.Halo("out"))
    for _ in range(3):
        S1 = st.mapstencil_(st.life, S1, steps=100, sync=False)
    torch.cuda.synchronize()
    S2 = st.SwitchingStencilArray(st.to_device(g), st.Moore(1), st.Wrap(), st.Halo("out"))
    S2 = st.mapstencil_(st.life, S2, steps=300)
    a = st.to_host(S1.source)[1:-1, 1:-1]
    b = st.to_host(S2.source)[1:-1, 1:-1]
    assert np.array_equal(a, b)


@pytest.mark.parametrize("n0", [33, 62, 63, 100, 1000, 4094])
@pytest.mark.parametrize("bname", ["wrap", "remove0"])
def test_life_ragged_rows(cuda, st, orc, abi, n0, bname):
    """Row lengths that are not a multiple of 32 take the packed path too (spare bits at the end of the
    column-interleaved rows, the two neighbours that fall on them replaced when read), persistent and
    multi-launch; both states bit-exact against the oracle, for B3/S23 and HighLife."""
    rng = np.random.default_rng(n0 + len(bname))
    n1 = 300 if n0 < 4000 else 160
    a = np.asfortranarray((rng.random((n0, n1)) < 0.35).astype(np.uint8))
    bnd = st.Wrap() if bname == "wrap" else st.Remove(0)
    for rule in (st.life, st.LifeRule((3, 6), (2, 3))):
        for steps in (1, 9, 40):
            S2, kern = _gpu_run(st, st.to_device(a), rule, bnd, st.Conditional(), steps)
            assert "life_coop" in kern or "life_block" in kern, kern
            res, prev, _ = _oracle_steps(orc, abi, st, a, abi.U8, rule, bnd, st.Conditional(), steps)
            assert np.array_equal(_logical(S2.source, st.Conditional(), st), res), (rule, steps)
            if steps > 1:
                assert np.array_equal(_logical(S2.dest, st.Conditional(), st), prev), (rule, steps)
