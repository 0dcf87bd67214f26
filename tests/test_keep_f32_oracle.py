"""The oracle's restatement of the STC_KEEP_F32 precision mode (CPU only): its stochastic BFloat16
rounding and its pass schedule."""
import numpy as np


def test_stochastic_rounding_properties(orc):
    rng = np.random.default_rng(0)
    x = np.asfortranarray(rng.random((64, 33, 5), dtype=np.float32))
    bits = orc.bf16_stochastic_bits(x, 12)
    lo = (x.view(np.uint32) >> 16).astype(np.uint16)
    # every result is one of the two BFloat16 neighbours of the input
    assert np.all((bits == lo) | (bits == lo + 1))
    # values already representable in BFloat16 are unchanged
    exact = orc.bf16_bits_to_f32(lo).reshape(x.shape, order="F")
    assert np.array_equal(orc.bf16_stochastic_bits(np.asfortranarray(exact), 3), lo)
    # unbiased on average: the mean rounding error is far below half a BFloat16 ulp
    up = orc.bf16_bits_to_f32(bits).reshape(x.shape)
    ulp = orc.bf16_bits_to_f32(lo + 1) - orc.bf16_bits_to_f32(lo)
    assert abs(float(np.mean((up - x) / ulp.reshape(x.shape)))) < 0.01
    # deterministic, and a different step gives different bits
    assert np.array_equal(bits, orc.bf16_stochastic_bits(x, 12))
    assert not np.array_equal(bits, orc.bf16_stochastic_bits(x, 13))
    # infinities and NaN round to nearest
    s = np.array([np.inf, -np.inf, np.nan], dtype=np.float32)
    assert np.array_equal(orc.bf16_stochastic_bits(s, 1), orc.f32_to_bf16_bits(s))


def test_keep_f32_schedule(orc):
    assert orc.keep_f32_schedule(1) == (0, 1)
    assert orc.keep_f32_schedule(4) == (0, 4)
    assert orc.keep_f32_schedule(5) == (1, 1)
    assert orc.keep_f32_schedule(8) == (1, 4)
    assert orc.keep_f32_schedule(9) == (2, 1)
    assert orc.keep_f32_schedule(200) == (49, 4)
    assert orc.keep_f32_schedule(200, 8) == (24, 8)
    assert orc.keep_f32_schedule(9, 8) == (1, 1)
