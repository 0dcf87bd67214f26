"""Remove's padval type on the GPU: maps whose padval promotes the neighbours
(promote_type(eltype, typeof(padval)), src/gatherstencil.jl:50) equal the oracle's restatement bit for bit,
multi-step runs convert each step back to the grid type, and a step whose result does not convert exactly
raises the reference's InexactError (STC_ERR_INEXACT)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["f32_f64pad_mean", "u8_half_sum", "i32_i64pad_max", "f32_f64pad_halo_mean",
                                  "bf16_f32pad_sum"])
def test_promoted_map_matches_oracle(cuda, st, orc, abi, case):
    import torch
    rng = np.random.default_rng(len(case))
    pad = st.Conditional()
    if case == "f32_f64pad_mean":
        a = np.asfortranarray(rng.random((130, 67), dtype=np.float32)); code = abi.F32
        red, hood, bnd = st.mean, st.Window(1), st.Remove(np.float64(0.1))
    elif case == "f32_f64pad_halo_mean":
        a = np.asfortranarray(rng.random((70, 45), dtype=np.float32)); code = abi.F32
        red, hood, bnd, pad = st.mean, st.Moore(1), st.Remove(np.float64(0.3)), st.Halo("out")
    elif case == "u8_half_sum":
        a = np.asfortranarray(rng.integers(0, 4, (90, 33)).astype(np.uint8)); code = abi.U8
        red, hood, bnd = st.sum, st.Window(1), st.Remove(0.5)
    elif case == "bf16_f32pad_sum":
        a = np.asfortranarray(rng.random((64, 40), dtype=np.float32)); code = abi.BF16
        red, hood, bnd = st.sum, st.VonNeumann(1), st.Remove(np.float32(0.25))
    else:
        a = np.asfortranarray(rng.integers(-50, 50, (77, 41)).astype(np.int32)); code = abi.I32
        red, hood, bnd = st.maximum, st.Circle(2), st.Remove(np.int64(60))
    if code == abi.BF16:
        d = st.colmajor_empty(a.shape, torch.bfloat16)
        d.copy_(st.to_device(a))
        from oracle.oracle import f32_to_bf16_bits
        host = np.asfortranarray(f32_to_bf16_bits(a))
    else:
        d = st.to_device(a)
        host = a
    sa = st.StencilArray(d, hood, bnd, pad)
    out = st.mapstencil(red, sa)
    parent = st.to_host(sa.parent) if code != abi.BF16 else np.asfortranarray(
        st.to_host(sa.parent.float()).astype(np.float32))
    if code == abi.BF16:
        from oracle.oracle import f32_to_bf16_bits
        parent = np.asfortranarray(f32_to_bf16_bits(parent))
    want = orc.map(parent if isinstance(pad, st.Halo) else host, code, hood, red, bnd, pad)
    got = st.to_host(out)
    assert got.dtype == want.dtype, (got.dtype, want.dtype)
    assert got.tobytes(order="F") == want.tobytes(order="F")


def test_promoted_steps_match_oracle(cuda, st, orc, abi):
    rng = np.random.default_rng(5)
    a = np.asfortranarray(rng.random((96, 50), dtype=np.float32))
    bnd = st.Remove(np.float64(0.1))
    S = st.SwitchingStencilArray(st.to_device(a), st.Window(1), bnd)
    S = st.mapstencil_(st.mean, S, steps=3)
    pa, pb = a.copy(order="F"), a.copy(order="F")
    in_b = orc.map_steps(pa, pb, abi.F32, st.Window(1), st.mean, bnd, st.Conditional(), 3)
    want, prev = (pb, pa) if in_b else (pa, pb)
    assert np.array_equal(st.to_host(S.source).view(np.uint32), want.view(np.uint32))
    assert np.array_equal(st.to_host(S.dest).view(np.uint32), prev.view(np.uint32))
    # Life on 0/1 UInt8 with an Int64 padval: promoted to Int64 and converted back exactly, so it equals the
    # UInt8 run
    g = np.asfortranarray((rng.random((64, 64)) < 0.3).astype(np.uint8))
    S1 = st.mapstencil_(st.life, st.SwitchingStencilArray(st.to_device(g), st.Moore(1), st.Remove(np.int64(0))), steps=5)
    S2 = st.mapstencil_(st.life, st.SwitchingStencilArray(st.to_device(g), st.Moore(1), st.Remove(0)), steps=5)
    assert np.array_equal(st.to_host(S1.source), st.to_host(S2.source))


def test_promoted_steps_inexact(cuda, st):
    """Sum of a UInt8 grid with Remove(0.5) is a Float64 with halves at the edges; storing it back into the
    UInt8 grid is the reference's InexactError."""
    from stencils_gb300._lib import StencilError
    a = np.ones((40, 30), dtype=np.uint8, order="F")
    S = st.SwitchingStencilArray(st.to_device(a), st.Window(1), st.Remove(0.5))
    with pytest.raises(StencilError) as e:
        st.mapstencil_(st.sum, S, steps=1)
    assert e.value.status == -13
    # the library's status word is clear again afterwards
    S = st.mapstencil_(st.sum, st.SwitchingStencilArray(st.to_device(a), st.Window(1), st.Remove(0)), steps=1)


def test_status_is_per_stream(cuda, st):
    """An inexact conversion queued without waiting on stream A is reported by the next synchronising
    call on stream A, not by a call that synchronises stream B in between."""
    import torch
    from stencils_gb300._lib import StencilError
    a = np.ones((40, 30), dtype=np.uint8, order="F")
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    with torch.cuda.stream(sa):
        S = st.SwitchingStencilArray(st.to_device(a), st.Window(1), st.Remove(0.5))
        st.mapstencil_(st.sum, S, steps=1, sync=False)          # queued; the error waits in A's slot
    with torch.cuda.stream(sb):
        T = st.SwitchingStencilArray(st.to_device(a), st.Window(1), st.Remove(0))
        st.mapstencil_(st.sum, T, steps=1)                      # B's own slot is clear
    with torch.cuda.stream(sa):
        U = st.SwitchingStencilArray(st.to_device(a), st.Window(1), st.Remove(0))
        with pytest.raises(StencilError) as e:
            st.mapstencil_(st.sum, U, steps=1)
        assert e.value.status == -13
        st.mapstencil_(st.sum, U, steps=1)                      # read once, then clear
