"""Temporally blocked 3D multi-step maps (K6): bit-exact against the oracle's per-step gather, the blocked
kernel is the one that ran, and the precision mode (STC_KEEP_F32) matches the oracle's restatement of it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_gpu(st, a, code, stencil, red, bnd, pad, steps):
    import torch
    from stencils_gb300 import _lib
    if code in ("bf16", "f16"):
        d = st.colmajor_empty(a.shape, torch.bfloat16 if code == "bf16" else torch.float16)
        d.copy_(st.to_device(a))
    else:
        d = st.to_device(a)
    S = st.SwitchingStencilArray(d, stencil, bnd, pad)
    _lib.profile_enable(True)
    S = st.mapstencil_(red, S, steps=steps)
    kern = _lib.profile_report()
    _lib.profile_enable(False)
    res = S.source.float().cpu().numpy() if code != "f32" else S.source.cpu().numpy()
    prev = S.dest.float().cpu().numpy() if code != "f32" else S.dest.cpu().numpy()
    if isinstance(pad, st.Halo):
        res, prev = res[1:-1, 1:-1, 1:-1], prev[1:-1, 1:-1, 1:-1]
    return np.asfortranarray(res), np.asfortranarray(prev), kern


def _run_oracle(st, orc, abi, a, code, stencil, red, bnd, steps):
    from oracle.oracle import f32_to_bf16_bits, bf16_bits_to_f32
    if code == "bf16":
        x = np.asfortranarray(f32_to_bf16_bits(a))
        c = abi.BF16
    elif code == "f16":
        x = np.asfortranarray(a.astype(np.float16))
        c = abi.F16
    else:
        x = np.asfortranarray(a)
        c = abi.F32
    pa, pb = x.copy(order="F"), x.copy(order="F")
    in_b = orc.map_steps(pa, pb, c, stencil, red, bnd, st.Conditional(), steps, nthreads=orc.max_threads())
    res, prev = (pb, pa) if in_b else (pa, pb)
    if code == "bf16":
        res, prev = bf16_bits_to_f32(res), bf16_bits_to_f32(prev)
    elif code == "f16":
        res, prev = res.astype(np.float32), prev.astype(np.float32)
    return np.asfortranarray(res), np.asfortranarray(prev)


@pytest.mark.parametrize("code", ["f32", "bf16", "f16"])
@pytest.mark.parametrize("bname", ["wrap", "remove0", "remove_half"])
@pytest.mark.parametrize("steps", [8, 9, 12, 15])
def test_diffusion_blocked_matches_oracle(cuda, st, orc, abi, monkeypatch, code, bname, steps):
    """The temporally blocked path (default for Float32 runs of 8 steps or more; 16-bit state takes it when
    forced): both states bit-exact against n separate maps of the oracle, on a grid whose x extent is not
    a multiple of the tile width."""
    if code != "f32":
        monkeypatch.setenv("STC_TBLOCK", "1")
    rng = np.random.default_rng(steps * 31 + len(bname))
    a = rng.random((200, 37, 29)).astype(np.float32)
    bnd = {"wrap": st.Wrap(), "remove0": st.Remove(0.0), "remove_half": st.Remove(0.5)}[bname]
    got, gprev, kern = _run_gpu(st, a, code, st.VonNeumann(1, 3), st.Diffusion(0.1), bnd, st.Conditional(), steps)
    assert "tblock3d" in kern
    want, wprev = _run_oracle(st, orc, abi, a, code, st.VonNeumann(1, 3), st.Diffusion(0.1), bnd, steps)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(gprev.view(np.uint32), wprev.view(np.uint32))   # state n-1 where the reference leaves it


@pytest.mark.parametrize("shape_name", ["moore_mean", "cross_sum", "vn_mean"])
def test_other_blocked_shapes_and_halo(cuda, st, orc, abi, shape_name):
    """VonNeumann mean and Cross sum take the blocked path (Conditional and Halo parents); Moore(1,3), whose
    taps include the corners of the planes above and below, takes the padded per-step path."""
    rng = np.random.default_rng(3)
    a = rng.random((68, 40, 35)).astype(np.float32)
    stencil, red = {"moore_mean": (st.Moore(1, 3), st.mean), "cross_sum": (st.Cross(1, 3), st.sum),
                    "vn_mean": (st.VonNeumann(1, 3), st.mean)}[shape_name]
    for pad in (st.Conditional(), st.Halo("out")):
        got, gprev, kern = _run_gpu(st, a, "f32", stencil, red, st.Wrap(), pad, 11)
        want, wprev = _run_oracle(st, orc, abi, a, "f32", stencil, red, st.Wrap(), 11)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), pad
        assert np.array_equal(gprev.view(np.uint32), wprev.view(np.uint32)), pad
        assert ("tblock3d" in kern) == (shape_name != "moore_mean"), kern


@pytest.mark.parametrize("code", ["bf16", "f16"])
@pytest.mark.parametrize("bname", ["wrap", "remove_half"])
@pytest.mark.parametrize("steps", [1, 3, 9, 10, 17])
def test_keep_f32_matches_oracle(cuda, st, orc, abi, code, bname, steps):
    """The precision mode (STC_KEEP_F32): Float32 inside passes of 8 (BFloat16) or 4 (Float16) steps,
    BFloat16 rounded stochastically from hashed bits at their ends; both states bit-exact against the
    oracle's restatement."""
    import torch
    from oracle.oracle import f32_to_bf16_bits
    rng = np.random.default_rng(steps + 5 * len(bname))
    a = rng.random((150, 33, 21)).astype(np.float32)
    bnd = {"wrap": st.Wrap(), "remove_half": st.Remove(0.5)}[bname]
    d = st.colmajor_empty(a.shape, torch.bfloat16 if code == "bf16" else torch.float16)
    d.copy_(st.to_device(a))
    S = st.SwitchingStencilArray(d, st.VonNeumann(1, 3), bnd)
    S = st.mapstencil_(st.Diffusion(0.1), S, steps=steps, keep_f32=True)
    x = np.asfortranarray(f32_to_bf16_bits(a)) if code == "bf16" else np.asfortranarray(a.astype(np.float16))
    want, wprev = orc.map_steps_keep_f32(x, abi.BF16 if code == "bf16" else abi.F16, st.VonNeumann(1, 3),
                                         st.Diffusion(0.1), bnd, st.Conditional(), steps, nthreads=orc.max_threads())
    got = np.asfortranarray(S.source.view(torch.int16).cpu().numpy()).view(np.uint16)
    gprev = np.asfortranarray(S.dest.view(torch.int16).cpu().numpy()).view(np.uint16)
    assert np.array_equal(got, np.asarray(want).view(np.uint16))
    assert np.array_equal(gprev, np.asarray(wprev).view(np.uint16))


def test_keep_f32_rejects_other_paths(cuda, st):
    """The precision mode runs only where the blocked path does: a 2D run returns STC_ERR_UNSUPPORTED."""
    import torch
    d = st.colmajor_empty((64, 64), torch.bfloat16)
    d.zero_()
    S = st.SwitchingStencilArray(d, st.Window(1), st.Wrap())
    with pytest.raises(NotImplementedError):
        st.mapstencil_(st.mean, S, steps=5, keep_f32=True)


def test_diffusion_512_cubed_mass_conserved(cuda, st):
    """The diffusion benchmark size: 512^3 Float32, Wrap, 200 steps through the default multi-step path; the FP64
    total of the grid (a conserved quantity for this scheme) drifts only by rounding."""
    import torch
    rng = np.random.Generator(np.random.PCG64(4))
    a = rng.random((512, 512, 512), dtype=np.float32)
    S = st.SwitchingStencilArray(st.to_device(a), st.VonNeumann(1, 3), st.Wrap())
    m0 = st.mass(S.source)
    S = st.mapstencil_(st.Diffusion(0.1), S, steps=200)
    torch.cuda.synchronize()
    m1 = st.mass(S.source)
    assert abs(m1 - m0) / m0 < 1e-6
    assert float(S.source.min()) >= 0.0 and float(S.source.max()) <= 1.0


@pytest.mark.parametrize("code", ["f32", "bf16"])
@pytest.mark.parametrize("bname", ["wrap", "reflect", "remove_half"])
@pytest.mark.parametrize("shape", [(72, 37, 29), (33, 20, 18)])
@pytest.mark.parametrize("steps", [4, 7])
def test_padded_multistep_matches_oracle(cuda, st, orc, abi, monkeypatch, code, bname, shape, steps):
    """Conditional 3D runs whose boundary needs edge patching go through the internal Halo-padded
    pair (ring refreshed every step); both states match the oracle bit for bit, including grids whose
    padded rows need pitch alignment."""
    rng = np.random.default_rng(steps * 7 + shape[0])
    a = rng.random(shape).astype(np.float32)
    bnd = {"wrap": st.Wrap(), "reflect": st.Reflect(), "remove_half": st.Remove(0.5)}[bname]
    got, gprev, kern = _run_gpu(st, a, code, st.VonNeumann(1, 3), st.Diffusion(0.1), bnd, st.Conditional(), steps)
    assert "halo_fill" in kern and "tblock3d" not in kern, kern
    want, wprev = _run_oracle(st, orc, abi, a, code, st.VonNeumann(1, 3), st.Diffusion(0.1), bnd, steps)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(gprev.view(np.uint32), wprev.view(np.uint32))


@pytest.mark.parametrize("stencil_name", ["moore_mean", "window_sum_r2"])
def test_padded_multistep_other_stencils(cuda, st, orc, abi, stencil_name):
    """Other 3D stencils (run-time offset table, radius 2) through the padded pair."""
    rng = np.random.default_rng(11)
    a = rng.random((40, 26, 21)).astype(np.float32)
    stencil, red = {"moore_mean": (st.Moore(1, 3), st.mean), "window_sum_r2": (st.Moore(2, 3), st.sum)}[stencil_name]
    got, gprev, kern = _run_gpu(st, a, "f32", stencil, red, st.Wrap(), st.Conditional(), 5)
    assert "halo_fill" in kern
    want, wprev = _run_oracle(st, orc, abi, a, "f32", stencil, red, st.Wrap(), 5)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(gprev.view(np.uint32), wprev.view(np.uint32))
