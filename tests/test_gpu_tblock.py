"""Temporally blocked 3D multi-step maps (plane-streaming wavefront): bit-exact against the oracle's
per-step gather, and the blocked kernel is the one that ran."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run_gpu(st, a, code, stencil, red, bnd, pad, steps):
    import torch
    from stencils_gb300 import _lib
    if code == "bf16":
        d = st.colmajor_empty(a.shape, torch.bfloat16)
        d.copy_(st.to_device(a))
    else:
        d = st.to_device(a)
    S = st.SwitchingStencilArray(d, stencil, bnd, pad)
    _lib.profile_enable(True)
    S = st.mapstencil_(red, S, steps=steps)
    kern = _lib.profile_report()
    _lib.profile_enable(False)
    res = S.source.float().cpu().numpy() if code == "bf16" else S.source.cpu().numpy()
    prev = S.dest.float().cpu().numpy() if code == "bf16" else S.dest.cpu().numpy()
    if isinstance(pad, st.Halo):
        res, prev = res[1:-1, 1:-1, 1:-1], prev[1:-1, 1:-1, 1:-1]
    return np.asfortranarray(res), np.asfortranarray(prev), kern


def _run_oracle(st, orc, abi, a, code, stencil, red, bnd, steps):
    from oracle.oracle import f32_to_bf16_bits, bf16_bits_to_f32
    if code == "bf16":
        x = np.asfortranarray(f32_to_bf16_bits(a))
        c = abi.BF16
    else:
        x = np.asfortranarray(a)
        c = abi.F32
    pa, pb = x.copy(order="F"), x.copy(order="F")
    in_b = orc.map_steps(pa, pb, c, stencil, red, bnd, st.Conditional(), steps, nthreads=orc.max_threads())
    res, prev = (pb, pa) if in_b else (pa, pb)
    if code == "bf16":
        res, prev = bf16_bits_to_f32(res), bf16_bits_to_f32(prev)
    return np.asfortranarray(res), np.asfortranarray(prev)


@pytest.mark.parametrize("code", ["f32", "bf16"])
@pytest.mark.parametrize("bname", ["wrap", "remove0", "remove_half"])
@pytest.mark.parametrize("steps", [3, 4, 9, 12])
def test_diffusion_blocked_matches_oracle(cuda, st, orc, abi, monkeypatch, code, bname, steps):
    monkeypatch.setenv("STC_NO_PADDED", "1")
    monkeypatch.setenv("STC_TBLOCK", "1")
    rng = np.random.default_rng(steps * 31 + len(bname))
    a = rng.random((72, 37, 29)).astype(np.float32)
    bnd = {"wrap": st.Wrap(), "remove0": st.Remove(0.0), "remove_half": st.Remove(0.5)}[bname]
    got, gprev, kern = _run_gpu(st, a, code, st.VonNeumann(1, 3), st.Diffusion(0.1), bnd, st.Conditional(), steps)
    assert "tblock3d" in kern
    want, wprev = _run_oracle(st, orc, abi, a, code, st.VonNeumann(1, 3), st.Diffusion(0.1), bnd, steps)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(gprev.view(np.uint32), wprev.view(np.uint32))   # state n-1 where the reference leaves it


@pytest.mark.parametrize("shape_name", ["moore_mean", "cross_sum", "vn_mean"])
def test_other_blocked_shapes_and_halo(cuda, st, orc, abi, monkeypatch, shape_name):
    monkeypatch.setenv("STC_NO_PADDED", "1")
    monkeypatch.setenv("STC_TBLOCK", "1")
    rng = np.random.default_rng(3)
    a = rng.random((68, 40, 35)).astype(np.float32)
    stencil, red = {"moore_mean": (st.Moore(1, 3), st.mean), "cross_sum": (st.Cross(1, 3), st.sum),
                    "vn_mean": (st.VonNeumann(1, 3), st.mean)}[shape_name]
    for pad in (st.Conditional(), st.Halo("out")):
        got, _, kern = _run_gpu(st, a, "f32", stencil, red, st.Wrap(), pad, 7)
        want, _ = _run_oracle(st, orc, abi, a, "f32", stencil, red, st.Wrap(), 7)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), pad
        if isinstance(pad, st.Conditional):
            assert "tblock3d" in kern


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
