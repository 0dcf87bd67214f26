"""Continuous-batching server: results equal the job run alone, jobs admitted while others run,
HBM-budget rejection, cancellation, and errors surfaced per job (host-side fault injection)."""
import math
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _job(st, rng, abi, kind=None):
    side = int(round(math.exp(rng.uniform(math.log(24), math.log(700)))))
    shape = (side, max(8, int(side * rng.uniform(0.6, 1.4))))
    kind = kind or ["f32", "bf16", "life"][int(rng.integers(3))]
    steps = int(rng.integers(1, 41))
    if kind == "life":
        a = (rng.random(shape) < 0.3).astype(np.uint8)
        return a, None, st.Moore(1), st.life, (st.Wrap() if rng.random() < 0.5 else st.Remove(0)), steps
    k5 = rng.standard_normal(25).astype(np.float32)
    red, hood = [(st.mean, st.Window(1)), (st.mean, st.Circle(3)), (st.sum, st.Cross(2)),
                 (st.kernelproduct, st.Kernel(st.Window(2), k5, weight_dtype="f32"))][int(rng.integers(4))]
    bnd = st.Wrap() if rng.random() < 0.5 else st.Remove(0.0)
    a = rng.random(shape).astype(np.float32)
    if kind == "bf16":
        from oracle.oracle import f32_to_bf16_bits
        if red is st.sum:
            red = st.mean
        return np.asfortranarray(f32_to_bf16_bits(a)), abi.BF16, hood, red, bnd, steps
    return a, None, hood, red, bnd, steps


def _alone(st, abi, a, code, hood, red, bnd, steps):
    import torch
    if code == abi.BF16:
        t = st.colmajor_empty(a.shape, torch.bfloat16)
        t.view(torch.int16).copy_(torch.from_numpy(np.asfortranarray(a).view(np.int16)))
    else:
        t = st.to_device(a)
    S = st.SwitchingStencilArray(t, hood, bnd, st.Conditional())
    S = st.mapstencil_(red, S, steps=steps)
    r = S.source
    if r.dtype == torch.bfloat16:
        return np.asfortranarray(r.view(torch.int16).cpu().numpy().view(np.uint16))
    return np.asfortranarray(r.cpu().numpy())


def test_results_same_alone_and_in_the_mix(cuda, st, abi):
    rng = np.random.default_rng(99)
    jobs = [_job(st, rng, abi) for _ in range(36)]
    ids = {}
    with st.Server(hbm_fraction=0.5, steps_per_tick=8) as srv:
        # a client thread submits with random gaps, so jobs arrive while others are on the GPU
        def client():
            for i, (a, code, hood, red, bnd, steps) in enumerate(jobs):
                ids[i] = srv.submit(a, hood, red, bnd, steps, code=code)
                time.sleep(float(rng.uniform(0, 0.004)))
        th = threading.Thread(target=client)
        th.start()
        th.join()
        srv.drain(120.0)
        stats = srv.stats()
        assert stats["finished"] == len(jobs) and stats["ticks"] >= 2
        for i, (a, code, hood, red, bnd, steps) in enumerate(jobs):
            got, lat = srv.fetch(ids[i])
            assert lat >= 0
            want = _alone(st, abi, a, code, hood, red, bnd, steps)
            assert np.array_equal(got, want), f"job {i}"


def test_budget_rejection_and_cancel(cuda, st, abi):
    from stencils_gb300._lib import StencilError
    rng = np.random.default_rng(1)
    with st.Server(hbm_fraction=1e-6, steps_per_tick=4) as srv:
        small = rng.random((32, 32)).astype(np.float32)       # 2 x 4 KiB fits
        big = rng.random((2048, 2048)).astype(np.float32)     # 2 x 16 MiB does not
        i_small = srv.submit(small, st.Window(1), st.mean, st.Wrap(), 5)
        i_big = srv.submit(big, st.Window(1), st.mean, st.Wrap(), 5)
        srv.drain(30.0)
        got, _ = srv.fetch(i_small)
        assert np.array_equal(got, _alone(st, abi, small, None, st.Window(1), st.mean, st.Wrap(), 5))
        with pytest.raises(StencilError) as e:
            srv.fetch(i_big)
        assert e.value.status == -9   # STC_ERR_BUDGET
    with st.Server(hbm_fraction=0.5, steps_per_tick=1) as srv:
        ids = [srv.submit(rng.random((512, 512)).astype(np.float32), st.Circle(3), st.mean, st.Wrap(), 400)
               for _ in range(3)]
        srv.cancel(ids[2])
        srv.cancel(ids[1])
        srv.drain(60.0)
        got, _ = srv.fetch(ids[0])
        assert got.shape == (512, 512)
        for i in ids[1:]:
            with pytest.raises(StencilError) as e:
                srv.fetch(i)
            assert e.value.status == -11   # STC_ERR_CANCELLED


def test_invalid_job_rejected_at_submit(cuda, st):
    from stencils_gb300._abi import ArgumentError
    with st.Server() as srv:
        with pytest.raises(ArgumentError):
            srv.submit(np.zeros((2, 40), np.float32), st.Window(3), st.mean, st.Wrap(), 3)   # radius >= axis
        with pytest.raises(NotImplementedError):
            srv.submit(np.zeros((40, 40), np.float64), st.Window(1), st.mean, st.Wrap(), 3)  # f64 not batched


def test_solo_lane_and_pitched_inputs(cuda, st, abi):
    """Grids of at least 2^21 cells run alone on the solo stream beside the ticks; inputs given as corners of a
    larger column-major array are copied from their pitched rows; every result equals the job run alone."""
    rng = np.random.default_rng(5)
    pool = np.asfortranarray(rng.random((1600, 1500), dtype=np.float32))
    jobs = [(pool[:1500, :1450], st.Window(1), st.mean, st.Wrap(), 9),        # solo, pitched
            (pool[:1450, :1500], st.VonNeumann(1), st.Diffusion(0.1), st.Remove(0.0), 13),   # solo, pitched
            (pool[:300, :200], st.Circle(3), st.mean, st.Wrap(), 20),         # tick lane, pitched
            (np.asfortranarray(pool[:257, :129]), st.Cross(2), st.sum, st.Remove(0.0), 7)]
    with st.Server(hbm_fraction=0.5, steps_per_tick=4) as srv:
        ids = [srv.submit(a, hood, red, bnd, steps) for a, hood, red, bnd, steps in jobs]
        srv.drain(120.0)
        assert sorted(srv.ready()) == sorted(ids)   # the completion queue reports each job once
        assert srv.ready() == []
        for i, (a, hood, red, bnd, steps) in zip(ids, jobs):
            got, _ = srv.fetch(i)
            want = _alone(st, abi, np.asfortranarray(a), None, hood, red, bnd, steps)
            assert np.array_equal(got, want)


def test_fetch_into_caller_buffer(cuda, st, abi):
    """stc_server_fetch (the copying form) writes the same result into the caller's memory as the zero-copy
    form, and the pinned buffer of the zero-copy form outlives the server."""
    import ctypes as C
    from stencils_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(8)
    a = np.asfortranarray(rng.random((300, 257)).astype(np.float32))
    want = _alone(st, abi, a, None, st.Window(1), st.mean, st.Wrap(), 12)
    with st.Server(hbm_fraction=0.5, steps_per_tick=4) as srv:
        i1 = srv.submit(a, st.Window(1), st.mean, st.Wrap(), 12)
        i2 = srv.submit(a, st.Window(1), st.mean, st.Wrap(), 12)
        srv.drain(60.0)
        out = np.empty_like(a, order="F")
        lat = C.c_double(0.0)
        rc = lib.stc_server_fetch(srv._h, i1, out.ctypes.data_as(C.c_void_p), out.nbytes, C.byref(lat))
        assert rc == 0 and lat.value >= 0
        assert np.array_equal(out, want)
        kept, _ = srv.fetch(i2)
    assert np.array_equal(kept, want)   # the server is gone; its pinned result is still readable
    del kept
