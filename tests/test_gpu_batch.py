"""The batched, graph-captured launch: every job bit-identical to running it alone, resident and
tiled jobs, several rounds with temporal blocking, the autotuner, and the plain sequential path."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _stencils(st, rng):
    k5 = rng.standard_normal(25).astype(np.float32)
    return [("mean", st.Window(1)), ("mean", st.Circle(3)), ("sum", st.Cross(2)),
            ("kdot", st.Kernel(st.Window(2), k5, weight_dtype="f32"))]


def _make_jobs(st, rng, n, side_lo, side_hi, max_steps, dtypes=("f32",)):
    import torch
    jobs = []
    for i in range(n):
        side = int(round(math.exp(rng.uniform(math.log(side_lo), math.log(side_hi)))))
        n0, n1 = side, max(8, int(side * rng.uniform(0.5, 1.5)))
        kind, hood = _stencils(st, rng)[int(rng.integers(4))]
        red = {"mean": st.mean, "sum": st.sum, "kdot": st.kernelproduct}[kind]
        bnd = st.Wrap() if rng.random() < 0.5 else st.Remove(0.0)
        dt = dtypes[int(rng.integers(len(dtypes)))]
        a = rng.random((n0, n1)).astype(np.float32)
        if dt == "life":
            a = (rng.random((n0, n1)) < 0.35).astype(np.uint8)
            hood, red, bnd = st.Moore(1), st.life, (st.Wrap() if rng.random() < 0.5 else st.Remove(0))
            dev = st.to_device(a)
        elif dt == "bf16":
            dev = st.to_device(a).to(torch.bfloat16)
            dev = st.colmajor_empty(a.shape, torch.bfloat16).copy_(dev)
            if kind == "sum":
                red = st.mean
        else:
            dev = st.to_device(a)
        steps = int(rng.integers(1, max_steps + 1))
        jobs.append((dev, hood, red, bnd, steps))
    return jobs


def _copy(st, t):
    c = st.colmajor_empty(tuple(t.shape), t.dtype, t.device)
    c.copy_(t)
    return c


def _alone(st, dev, hood, red, bnd, steps):
    S = st.SwitchingStencilArray(_copy(st, dev), hood, bnd, st.Conditional())
    S = st.mapstencil_(red, S, steps=steps)
    return S.source.cpu()


@pytest.mark.parametrize("autotune", [False, True])
def test_batch_equals_alone(cuda, st, autotune):
    import torch
    rng = np.random.default_rng(17 + autotune)
    jobs = _make_jobs(st, rng, 40, 16, 600, 20, dtypes=("f32", "bf16", "life"))
    # a few large grids to force the tiled path with several rounds
    jobs += _make_jobs(st, np.random.default_rng(3), 4, 700, 900, 13)
    b = st.Batch()
    arrays = []
    for dev, hood, red, bnd, steps in jobs:
        S = st.SwitchingStencilArray(_copy(st, dev), hood, bnd, st.Conditional())
        arrays.append(S)
        b.add(red, S, steps)
    b.plan(autotune=autotune)
    b.run()
    torch.cuda.synchronize()
    for i, (dev, hood, red, bnd, steps) in enumerate(jobs):
        got = b.result(i).source.cpu()
        want = _alone(st, dev, hood, red, bnd, steps)
        assert torch.equal(got.view(torch.uint8) if got.dtype == torch.bool else got,
                           want.view(torch.uint8) if want.dtype == torch.bool else want), f"job {i}"
    b.close()


def test_batch_replay_and_sequential(cuda, st):
    """The captured graph replays (each replay continues from the previous result); the plain
    sequential path (one synchronising mapstencil_ loop per job) reaches the same states."""
    import torch
    rng = np.random.default_rng(5)
    jobs = _make_jobs(st, rng, 12, 32, 400, 9)
    b = st.Batch()
    seq = st.Batch()
    pairs = []
    for dev, hood, red, bnd, steps in jobs:
        S1 = st.SwitchingStencilArray(_copy(st, dev), hood, bnd, st.Conditional())
        S2 = st.SwitchingStencilArray(_copy(st, dev), hood, bnd, st.Conditional())
        b.add(red, S1, steps)
        seq.add(red, S2, steps)
        pairs.append((S1, S2, dev, hood, red, bnd, steps))
    b.plan(autotune=False)
    b.run()
    torch.cuda.synchronize()
    first = [b.result(i).source.clone() for i in range(len(pairs))]
    # second replay: start from the first results, copied back into the source parents
    for i, (S1, *_rest) in enumerate(pairs):
        S1.source.copy_(first[i])
    b.run()
    seq.run_sequential()
    torch.cuda.synchronize()
    for i, (S1, S2, dev, hood, red, bnd, steps) in enumerate(pairs):
        want1 = _alone(st, dev, hood, red, bnd, steps)
        assert torch.equal(first[i].cpu(), want1)
        want2 = _alone(st, want1.cuda(), hood, red, bnd, steps)
        assert torch.equal(b.result(i).source.cpu(), want2)
        seq_res = S2.source if steps % 2 == 0 else S2.dest
        assert torch.equal(seq_res.cpu(), want1)
    b.close()
    seq.close()


def test_batch_life_resident_and_tiled_match_oracle(cuda, st, orc, abi):
    import torch
    rng = np.random.default_rng(8)
    b = st.Batch()
    cases = []
    for shape, steps in (((96, 64), 33), ((1024, 512), 21)):
        a = (rng.random(shape) < 0.3).astype(np.uint8)
        S = st.SwitchingStencilArray(st.to_device(a), st.Moore(1), st.Wrap(), st.Conditional())
        b.add(st.life, S, steps)
        cases.append((a, steps))
    b.plan(autotune=False)
    b.run()
    torch.cuda.synchronize()
    for i, (a, steps) in enumerate(cases):
        pa, pb = np.asfortranarray(a), np.asfortranarray(a.copy())
        in_b = orc.map_steps(pa, pb, abi.U8, st.Moore(1), st.life, st.Wrap(), st.Conditional(), steps,
                             nthreads=orc.max_threads())
        want = pb if in_b else pa
        got = np.asfortranarray(b.result(i).source.cpu().numpy())
        assert np.array_equal(got, want)
    b.close()
