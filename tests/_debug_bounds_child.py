"""Child process of test_gpu_debug_bounds.py, started with STC_DEBUG_BOUNDS=1 so the package loads
libstencilcuda_debug.so (the kernels' device-side bounds tests compiled in).  Runs small odd-sized grids —
one cell more than the radius up to a few cells past two radii, per axis — through single maps, multi-step
runs (blocked and per-step), Life (packed, rows with and without spare bits) and the batch, compares each
with the oracle bit for bit, and fails on the first mismatch or STC_ERR_BOUNDS (the call raises)."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import numpy as np  # noqa: E402

import __graft_entry__ as entry  # noqa: E402

st = entry.load_package()
import stencils_gb300._abi as A  # noqa: E402
from stencils_gb300 import _lib  # noqa: E402
from oracle import oracle as orc  # noqa: E402
from _backends import GpuBackend, OracleBackend  # noqa: E402

lib = _lib.load()
assert lib.stc_debug_bounds() == 1, "not the debug build"
gpu, ora = GpuBackend(st, A), OracleBackend(st, orc, A)
rng = np.random.default_rng(11)
n = 0


def same(x, y, what):
    global n
    x, y = np.asarray(x), np.asarray(y)
    assert x.shape == y.shape and x.tobytes(order="F") == y.tobytes(order="F"), what
    n += 1


# single maps: named shapes (specialised and vector kernels) and an offset table
hoods = [st.Window(1), st.Moore(1), st.VonNeumann(1), st.Circle(3), st.Cross(2), st.Annulus(3, 1)]
for hood in hoods:
    R = hood.radius
    for shape in ((R + 1, R + 1), (R + 2, 2 * R + 3), (2 * R + 3, R + 1), (2 * R + 37, 3 * R + 5)):
        for bnd in (st.Remove(0.0), st.Wrap(), st.Reflect()):
            for pad in (st.Conditional(), st.Halo("out")):
                a = np.asfortranarray(rng.random(shape).astype(np.float32))
                same(gpu.map(a, hood, st.mean, bnd, pad), ora.map(a, hood, st.mean, bnd, pad), (hood, shape, bnd, pad))
# 3D maps and multi-step runs
for shape in ((2, 2, 2), (3, 4, 5), (9, 7, 6)):
    a = np.asfortranarray(rng.random(shape).astype(np.float32))
    for bnd in (st.Wrap(), st.Remove(0.5)):
        same(gpu.switch_map(a, st.VonNeumann(1, 3), st.Diffusion(0.1), bnd, st.Conditional(), steps=9),
             ora.switch_map(a, st.VonNeumann(1, 3), st.Diffusion(0.1), bnd, st.Conditional(), steps=9), (shape, bnd))
# 2D multi-step runs: the blocked path (17 steps) on grids smaller than one box, and per-step runs
for shape in ((2, 2), (3, 5), (7, 130), (131, 6)):
    a = np.asfortranarray(rng.random(shape).astype(np.float32))
    for hood, red in ((st.Window(1), st.mean), (st.VonNeumann(1), st.Diffusion(0.1))):
        for bnd in (st.Wrap(), st.Remove(0.25)):
            same(gpu.switch_map(a, hood, red, bnd, st.Conditional(), steps=17),
                 ora.switch_map(a, hood, red, bnd, st.Conditional(), steps=17), (shape, hood, bnd))
# Life: packed rows with and without spare bits, bands shorter than the ghost depth
for shape in ((32, 2), (33, 2), (64, 3), (95, 5), (128, 7), (4096, 3)):
    a = np.asfortranarray((rng.random(shape) < 0.4).astype(np.uint8))
    for bnd in (st.Wrap(), st.Remove(0)):
        for steps in (1, 2, 11):
            same(gpu.switch_map(a, st.Moore(1), st.life, bnd, st.Conditional(), steps=steps),
                 ora.switch_map(a, st.Moore(1), st.life, bnd, st.Conditional(), steps=steps), (shape, bnd, steps))
# the batch: resident and tiled jobs of odd sizes
b = st.Batch()
jobs = []
for shape in ((3, 3), (5, 9), (130, 67), (300, 131)):
    a = np.asfortranarray(rng.random(shape).astype(np.float32))
    S = st.SwitchingStencilArray(st.to_device(a), st.Window(1), st.Wrap(), st.Conditional())
    b.add(st.mean, S, 5)
    jobs.append(a)
b.plan(autotune=False)
b.run()
for i, a in enumerate(jobs):
    same(st.to_host(b.result(i).source), ora.switch_map(a, st.Window(1), st.mean, st.Wrap(), st.Conditional(), steps=5), i)
print("ok", n)
