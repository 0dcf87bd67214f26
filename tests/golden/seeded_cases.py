"""Seeded parity cases, one per benchmark configuration and per extra path, at sizes the oracle runs in
milliseconds.  `make_seeded_fixtures.py` runs each case on the oracle and commits the inputs and outputs
under `seeded/` as raw column-major binaries with a manifest; `tests/test_seeded_fixtures.py` checks the
oracle (CPU suite) and the GPU library (GPU suite) against those files.

Each case states the reference call it restates in Julia syntax (`julia`), so a host with Julia and the
reference can run the same inputs: `seeded/run_reference.jl` reads the manifest and the binaries.

Inputs come from numpy's PCG64 with the configuration's seed and distribution (Julia's own generator
cannot be reproduced here); the binaries carry them exactly.
"""
from __future__ import annotations

import math
import operator
from dataclasses import dataclass
from typing import Callable

import numpy as np


@dataclass
class Case:
    name: str
    description: str
    julia: str
    make_inputs: Callable          # (st, abi) -> dict name -> (array, abi code)
    run: Callable                  # (mode, st, abi, orc, inputs) -> (array, abi code); mode "oracle" | "gpu"
    tolerance: str = "bit-exact"   # or "kdot-f32": |gpu - oracle| <= 2 L 2^-24 sum|w v| (+ one bf16 rounding)


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def gauss_weights(st):
    """Kernel(Window(3)) normalised Gaussian, sigma 1.5, over the stencil's distances (Float64)."""
    w = np.array([math.exp(-d * d / (2 * 1.5 ** 2)) for d in st.Window(3).distances()])
    return w / w.sum()


# ------------------------------------------------------------------ runners shared by the cases
def _backend(mode, st, abi, orc):
    import sys
    from pathlib import Path
    tests_dir = str(Path(__file__).resolve().parents[1])
    if tests_dir not in sys.path:
        sys.path.insert(0, tests_dir)
    from _backends import GpuBackend, OracleBackend
    return OracleBackend(st, orc, abi) if mode == "oracle" else GpuBackend(st, abi)


def _map_runner(stencil_fn, red_fn, bnd_fn, pad_fn, out_code=None):
    def run(mode, st, abi, orc, inputs):
        a, code = inputs["A"]
        stencil = stencil_fn(st, inputs)
        out = _backend(mode, st, abi, orc).map(a, stencil, red_fn(st), bnd_fn(st), pad_fn(st), code=code)
        return out, (code if out_code is None else out_code(abi))
    return run


def _switch_runner(stencil_fn, red_fn, bnd_fn, pad_fn, steps):
    def run(mode, st, abi, orc, inputs):
        a, code = inputs["A"]
        out = _backend(mode, st, abi, orc).switch_map(a, stencil_fn(st, inputs), red_fn(st), bnd_fn(st),
                                                      pad_fn(st), steps=steps, code=code)
        return out, code
    return run


def _gauss_kernel(st, inputs):
    w, _ = inputs["weights"]
    return st.Kernel(st.Window(3), w.astype(np.float32), weight_dtype="f32")


# ------------------------------------------------------------------ inputs
def _in_mean_blur(st, abi):
    return {"A": (np.asfortranarray(_rng(1).random((40, 30))), abi.F64)}


def _in_life(st, abi):
    return {"A": (np.asfortranarray((_rng(2).random((64, 64)) < 0.3).astype(np.uint8)), abi.U8)}


def _in_gauss(st, abi, bf16=False):
    a = np.asfortranarray(_rng(3).random((48, 40), dtype=np.float32))
    w = gauss_weights(st).astype(np.float32)
    if bf16:
        from oracle.oracle import f32_to_bf16_bits
        return {"A": (np.asfortranarray(f32_to_bf16_bits(a)), abi.BF16), "weights": (w, abi.F32)}
    return {"A": (a, abi.F32), "weights": (w, abi.F32)}


def _in_diffusion(st, abi):
    return {"A": (np.asfortranarray(_rng(4).random((12, 12, 12), dtype=np.float32)), abi.F32)}


def _in_reflect_circle(st, abi):
    return {"A": (np.asfortranarray(_rng(9).random((36, 28), dtype=np.float32)), abi.F32)}


def _in_terms(st, abi):
    r = _rng(7)
    a = np.asfortranarray(r.random((32, 24)))
    b = np.asfortranarray(r.random((32, 24)))
    return {"A": (a, abi.F64), "B": (b, abi.F64)}


def _in_scatter(st, abi):
    r = _rng(8)
    # 21 columns, a multiple of 2R + 1: the reference's threaded passes then never meet at the Wrap seam
    return {"A": (np.asfortranarray(r.random((30, 21))), abi.F64),
            "dest0": (np.asfortranarray(r.random((30, 21))), abi.F64)}


def _in_layered(st, abi):
    return {"A": (np.asfortranarray(_rng(10).random((30, 22)) * 2 - 1), abi.F64)}


# ------------------------------------------------------------------ multi-array, scatter, Layered runners
def _run_terms(mode, st, abi, orc, inputs):
    a, _ = inputs["A"]
    b, _ = inputs["B"]
    f = st.Terms(st.center, st.scaled(0.1, st.sum))
    if mode == "oracle":
        items = [(a.copy(order="F"), st.Moore(1), st.Remove(0.0), st.Conditional()),
                 (b.copy(order="F"), st.Moore(1), st.Remove(0.0), st.Conditional())]
        return orc.map_terms(f, items, abi.F64), abi.F64
    sa = st.StencilArray(st.to_device(a), st.Moore(1), st.Remove(0.0))
    sb = st.StencilArray(st.to_device(b), st.Moore(1), st.Remove(0.0))
    return st.to_host(st.mapstencil(f, sa, sb)), abi.F64


def _run_scatter(mode, st, abi, orc, inputs):
    a, _ = inputs["A"]
    d0, _ = inputs["dest0"]
    if mode == "oracle":
        return orc.scatter(st.scatter_center, operator.add, d0.copy(order="F"), a.copy(order="F"), abi.F64,
                           st.Moore(1), st.Wrap(), st.Conditional()), abi.F64
    dest = st.to_device(d0)
    st.scatterstencil_(st.scatter_center, operator.add, dest, st.StencilArray(st.to_device(a), st.Moore(1), st.Wrap()))
    return st.to_host(dest), abi.F64


def _layered(st):
    return st.Layered(x=st.Layered(a=st.Moore(1), b=st.Window(2)), y=st.Circle(3))


def _run_layered(mode, st, abi, orc, inputs):
    from stencils_gb300.stencil import with_radius
    a, _ = inputs["A"]
    L = _layered(st)
    f = st.Terms(st.mean, None, st.scaled(0.5, st.sum))
    if mode == "oracle":
        items = [(a.copy(order="F"), with_radius(l, L.radius), st.Wrap(), st.Conditional()) for l in L.leaves()]
        return orc.map_terms(f, items, abi.F64), abi.F64
    sa = st.StencilArray.from_parent(st.to_device(a), L, st.Wrap(), st.Conditional())
    return st.to_host(st.mapstencil(f, sa)), abi.F64


# ------------------------------------------------------------------ the cases
CASES = [
    Case("mean_blur_f64",
         "mean blur: Window(1) mean, Float64 U[0,1) seed 1, Remove(0.0), Conditional (the 1000x1000 "
         "configuration's shape and distribution at 40x30)",
         "mapstencil(mean, StencilArray(A, Window(1); boundary=Remove(0.0), padding=Conditional()))",
         _in_mean_blur,
         _map_runner(lambda st, i: st.Window(1), lambda st: st.mean, lambda st: st.Remove(0.0),
                     lambda st: st.Conditional())),
    Case("life_u8",
         "Conway's Life B3/S23 on UInt8 Bernoulli(0.3) seed 2, Moore(1), Wrap, Halo{:out}, "
         "SwitchingStencilArray, 10 generations (the 4096x4096 configuration at 64x64)",
         "life(h) = (s = sum(neighbors(h)); UInt8(s == 3 || (center(h) == 1 && s == 2))); "
         "S = SwitchingStencilArray(A, Moore(1); boundary=Wrap(), padding=Halo{:out}()); "
         "for _ in 1:10; S = mapstencil!(life, S); end; parent(S)[2:end-1, 2:end-1]",
         _in_life,
         _switch_runner(lambda st, i: st.Moore(1), lambda st: st.life, lambda st: st.Wrap(),
                        lambda st: st.Halo("out"), 10)),
    Case("gauss7_f32",
         "7x7 Gaussian kernelproduct, Kernel(Window(3)) sigma 1.5 normalised (Float32 weights), Float32 "
         "U[0,1) seed 3, Remove(0f0) (the 8192x8192 configuration at 48x40)",
         "mapstencil(kernelproduct, StencilArray(A, Kernel(Window(3), SVector{49}(weights)); "
         "boundary=Remove(0f0)))",
         lambda st, abi: _in_gauss(st, abi),
         _map_runner(_gauss_kernel, lambda st: st.kernelproduct, lambda st: st.Remove(0.0),
                     lambda st: st.Conditional()),
         tolerance="kdot-f32"),
    Case("gauss7_bf16",
         "the 7x7 Gaussian with BFloat16 storage (the Float32 inputs rounded to BFloat16), Float32 weights "
         "and accumulation, BFloat16 result",
         "mapstencil(kernelproduct, StencilArray(A_bf16, Kernel(Window(3), SVector{49}(weights)); "
         "boundary=Remove(BFloat16(0)))) with the fold in Float32 and one rounding to BFloat16",
         lambda st, abi: _in_gauss(st, abi, bf16=True),
         _map_runner(_gauss_kernel, lambda st: st.kernelproduct, lambda st: st.Remove(0.0),
                     lambda st: st.Conditional()),
         tolerance="kdot-f32"),
    Case("diffusion3d_f32",
         "explicit 3D diffusion c + 0.1f0 (sum - 6c) over VonNeumann(1, 3), Float32 U[0,1) seed 4, Wrap, "
         "SwitchingStencilArray, 5 steps (the 512^3 configuration at 12^3)",
         "diffuse(h) = center(h) + 0.1f0 * (sum(neighbors(h)) - 6 * center(h)); "
         "S = SwitchingStencilArray(A, VonNeumann(1, 3); boundary=Wrap()); "
         "for _ in 1:5; S = mapstencil!(diffuse, S); end; parent(S)",
         _in_diffusion,
         _switch_runner(lambda st, i: st.VonNeumann(1, 3), lambda st: st.Diffusion(0.1), lambda st: st.Wrap(),
                        lambda st: st.Conditional(), 5)),
    Case("circle3_reflect_f32",
         "Circle(3) mean, Float32 U[0,1) seed 9, Reflect, Halo{:out}",
         "mapstencil(mean, StencilArray(A, Circle(3); boundary=Reflect(), padding=Halo{:out}()))",
         _in_reflect_circle,
         _map_runner(lambda st, i: st.Circle(3), lambda st: st.mean, lambda st: st.Reflect(),
                     lambda st: st.Halo("out"))),
    Case("two_array_f64",
         "maps over two arrays: center(A) + 0.1 * sum(neighbors(B)), Moore(1), Remove(0.0) on both, "
         "Float64 U[0,1) seed 7 (A then B from one stream)",
         "mapstencil((a, b) -> center(a) + 0.1 * sum(b), StencilArray(A, Moore(1); boundary=Remove(0.0)), "
         "StencilArray(B, Moore(1); boundary=Remove(0.0)))",
         _in_terms, _run_terms),
    Case("scatter_center_f64",
         "scatterstencil! of each cell's centre value to its Moore(1) neighbours with +, Wrap, onto a "
         "random Float64 dest (seed 8: source then dest)",
         "scatterstencil!(h -> map(_ -> center(h), neighbors(h)), +, dest0, StencilArray(A, Moore(1); "
         "boundary=Wrap()))",
         _in_scatter, _run_scatter),
    Case("layered_f64",
         "a Layered stencil (x = Layered(a = Moore(1), b = Window(2)), y = Circle(3)) mapped with "
         "mean(l.x.a) + 0.5 * sum(l.y), Float64 U[-1,1) seed 10, Wrap",
         "mapstencil(l -> mean(l.x.a) + 0.5 * sum(l.y), StencilArray(A, Layered(x=Layered(a=Moore(1), "
         "b=Window(2)), y=Circle(3)); boundary=Wrap()))",
         _in_layered, _run_layered),
]

BY_NAME = {c.name: c for c in CASES}
