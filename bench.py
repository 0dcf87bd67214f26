"""Benchmark of the mapstencil hot path on GB300 (one JSON line on rank 0).

Workload (one "step"): Conway's Life on a 4096x4096 UInt8 grid, initial density 0.3 Bernoulli from
seed 2, Moore(1) B3/S23, Wrap boundary, Halo padding, SwitchingStencilArray: 1000 generations of
`A = mapstencil!(life, A)`.  Inputs are synthetic (seeded numpy PCG64).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`value`      whole-job Gcell-updates/s with the state resident in HBM (device-timed, CUDA events,
             L2 flushed between timed steps by writing a 256 MiB buffer).
`e2e`        the same metric through the public API with host (pinned) buffers: every step copies
             the initial grid host->device, runs the 1000 generations, and copies the result back.
`roofline`   the dominant kernel's algorithmic bytes (1 B read + 1 B written per cell update) per
             launch over its CUDA-event launch time, against the measured HBM copy bandwidth.
`cpu_baseline` the oracle (a C restatement of the reference's gather, OpenMP; for Moore(1) Life on
             UInt8 Halo parents the specialised loop the reference's compiled kernel amounts to) on
             the host cores, on a bounded number of generations of the same grid.
--impl reference times that CPU implementation as the reference arm (rank 0 only).
N > 1 runs N independent replicas (the path has no data exchange between GPUs).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__ as entry  # noqa: E402

METRIC = "Gcell-updates/s, % of HBM roofline; served p50/p99 latency vs plain mapstencil"
UNIT = "Gcell-updates/s"
SIDE = 4096
GENERATIONS = 1000
SEED = 2
DENSITY = 0.3
CONFIG = {"workload": "Conway Life B3/S23, Moore(1), UInt8 4096x4096, Wrap boundary, Halo padding, "
                      "SwitchingStencilArray 1000 generations per step",
          "grid": [SIDE, SIDE], "dtype": "u8", "generations_per_step": GENERATIONS,
          "initial_density": DENSITY, "seed": SEED, "l2": "flushed between timed steps (256 MiB write)"}


def initial_grid() -> np.ndarray:
    rng = np.random.Generator(np.random.PCG64(SEED))
    return np.asfortranarray((rng.random((SIDE, SIDE)) < DENSITY).astype(np.uint8))


# ------------------------------------------------------------------ distributed helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def init_dist(backend):
    import torch.distributed as dist
    ws, rank, _ = dist_env()
    if ws > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return ws, rank


def max_over_ranks(x: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not dist.is_initialized():
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    import torch.distributed as dist
    if dist.is_initialized():
        dist.barrier()


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def wait_first(self, timeout_s: float):
        """Block until the sampler has produced its first line (or timeout_s passes)."""
        t0 = time.perf_counter()
        while self.proc is not None and not self.lines and time.perf_counter() - t0 < timeout_s:
            time.sleep(0.02)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline (oracle)
def cpu_life_rate(target_s: float, threads: int | None = None):
    """Time the oracle's Life on the full grid for enough generations to take ~target_s seconds."""
    from oracle import oracle as orc
    st = entry.load_package()
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    threads = threads or orc.max_threads()
    a0 = initial_grid()
    pa = np.zeros((SIDE + 2, SIDE + 2), dtype=np.uint8, order="F")
    pa[1:-1, 1:-1] = a0
    pb = pa.copy(order="F")
    t0 = time.perf_counter()
    orc.map_steps(pa, pb, A.U8, st.Moore(1), st.life, st.Wrap(), st.Halo("in"), 1, nthreads=threads)
    t1 = time.perf_counter() - t0
    gens = max(1, int(round(target_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    orc.map_steps(pa, pb, A.U8, st.Moore(1), st.life, st.Wrap(), st.Halo("in"), gens, nthreads=threads)
    dt = time.perf_counter() - t0
    rate = gens * SIDE * SIDE / dt / 1e9
    return rate, threads, gens, dt


def run_reference(args):
    """The reference arm: the CPU implementation of the path (the oracle) on the host cores."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as orc
    orc.build()
    # calibrate a bounded sample: generations per step so that one step takes about 3 s, less when many
    # steps are asked for (the whole run stays near a minute)
    per_step = min(3.0, max(0.2, 60.0 / max(1, args.warmup + args.steps)))
    _, threads, _, _ = cpu_life_rate(0.5)
    rate1, _, gens, _ = cpu_life_rate(per_step, threads)
    st = entry.load_package()
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    a0 = initial_grid()
    pa = np.zeros((SIDE + 2, SIDE + 2), dtype=np.uint8, order="F")
    pa[1:-1, 1:-1] = a0
    pb = pa.copy(order="F")
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        orc.map_steps(pa, pb, A.U8, st.Moore(1), st.life, st.Wrap(), st.Halo("in"), gens, nthreads=threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = args.steps * gens * SIDE * SIDE / total / 1e9
    sample = (f"{gens} generations of the 4096x4096 grid per step, OpenMP {threads} threads, "
              "specialised Moore(1) loop")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": CONFIG,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "CPU restatement of the reference's gather (oracle/stencil_oracle.c: a vectorised Moore(1) "
                    "loop reading the Halo parent directly, as the reference's kernel specialised on the stencil "
                    "type does); the reference is "
                    "Julia and no julia binary exists on this host"}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm
def run_gpu(args):
    import torch
    ws, rank = init_dist("nccl" if int(os.environ.get("WORLD_SIZE", "1")) > 1 else "gloo")
    _, _, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    entry.build()
    st = entry.load_package()
    from stencils_gb300 import _lib
    _lib.load()

    a0 = initial_grid()
    S = st.SwitchingStencilArray(st.to_device(a0, dev), st.Moore(1), st.Wrap(), st.Halo("out"))
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream()
    updates_per_step = GENERATIONS * SIDE * SIDE

    for _ in range(args.warmup):
        S = st.mapstencil_(st.life, S, steps=GENERATIONS, sync=False)
    torch.cuda.synchronize()

    def timed_pass(profile: bool):
        """K steps bracketed by barrier + synchronize; device seconds of the steps (CUDA events).
        The calls are queued without waiting (sync=False), so the host's call overhead overlaps the
        GPU's work instead of showing up as idle time between the events."""
        nonlocal S
        barrier()
        torch.cuda.synchronize()
        _lib.profile_enable(profile)
        evs = []
        for _ in range(args.steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            S = st.mapstencil_(st.life, S, steps=GENERATIONS, sync=False)
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        prof = _lib.profile_report() if profile else {}
        _lib.profile_enable(False)
        barrier()
        return sum(a.elapsed_time(b) for a, b in evs) / 1e3, prof

    # value: the timed region without per-launch events; the roofline's per-launch durations come from
    # a second pass of the same K steps with an event pair around every library launch
    clocks = ClockSampler(local)
    clocks.start()
    clocks.wait_first(3.0)
    t_wall0 = time.perf_counter()
    dev_s, _ = timed_pass(False)
    wall = time.perf_counter() - t_wall0
    _, prof = timed_pass(True)
    dev_s_max = max_over_ranks(dev_s, dev)
    value = ws * args.steps * updates_per_step / dev_s_max / 1e9

    # roofline of the dominant kernel
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    dom = max(prof.items(), key=lambda kv: kv[1]["ms"]) if prof else (None, None)
    roof = None
    launches = sum(v["launches"] for v in prof.values())
    if dom[0]:
        k = dom[1]
        achieved = k["alg_bytes"] / (k["ms"] / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": dom[0], "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_src, "traffic": None,
                "launches": k["launches"], "avg_launch_us": 1e3 * k["ms"] / k["launches"],
                "alg_bytes_per_launch": k["alg_bytes"] / k["launches"],
                "updates_per_launch": k["updates"] / k["launches"],
                "share_of_device_time": k["ms"] / max(1e-9, sum(v["ms"] for v in prof.values()))}
        tfile = ROOT / "profiles" / "traffic.json"
        if tfile.exists():
            t = json.loads(tfile.read_text()).get(dom[0])
            if t:
                roof["traffic"] = t["bytes_per_launch"]
                roof["traffic_source"] = t["source"]

    # e2e through the public API with pinned host buffers
    pinned_in = torch.empty((SIDE, SIDE), dtype=torch.uint8).pin_memory()
    pinned_in.copy_(torch.from_numpy(np.ascontiguousarray(a0.T)))
    pinned_out = torch.empty((SIDE, SIDE), dtype=torch.uint8).pin_memory()
    S2 = st.SwitchingStencilArray(st.to_device(a0, dev), st.Moore(1), st.Wrap(), st.Halo("out"))
    e2e_times = []
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        # source parent interior <- host (column-major grid == row-major transpose); the three stages
        # are queued in stream order and the step ends when the result is in pinned host memory
        S2.source[1:-1, 1:-1].T.copy_(pinned_in, non_blocking=True)
        S2 = st.mapstencil_(st.life, S2, steps=GENERATIONS, sync=False)
        pinned_out.copy_(S2.source[1:-1, 1:-1].T, non_blocking=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_times.append(dt)
    # the clock record spans the three timed passes (device-timed, per-launch-traced, end to end)
    clk = clocks.stop()
    e2e_s = max_over_ranks(sum(e2e_times), dev)
    e2e_value = ws * args.steps * updates_per_step / e2e_s / 1e9

    if rank != 0:
        return 0
    cpu = None
    if not args.no_cpu_baseline:
        rate, threads, gens, dt = cpu_life_rate(args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{gens} generations of the 4096x4096 grid ({dt:.1f} s), oracle OpenMP {threads} threads, "
                         "specialised Moore(1) loop"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": CONFIG,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": SIDE * SIDE,
                    "d2h_bytes_per_step": SIDE * SIDE},
            "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
            "kernels": prof, "wall_s_timed_region": wall}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ the other benchmark workloads
def _timed_steps(fn, steps, warmup, flush):
    """Device time of `steps` calls of fn(), L2 flushed (outside the timing) before each; fn queues its
    work without waiting and the steps are queued back to back (one synchronisation at the end), so
    the events time the GPU's work rather than host call overhead wherever the host keeps ahead."""
    import torch
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    evs = []
    for _ in range(steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in evs) / 1e3


def _kernel_roofline(prof, peak_gbs):
    dom = max(prof.items(), key=lambda kv: kv[1]["ms"])
    k = dom[1]
    ach = k["alg_bytes"] / (k["ms"] / 1e3) / 1e9
    return {"kernel": dom[0], "achieved_gbs": ach, "frac_of_measured_hbm": ach / peak_gbs,
            "avg_launch_us": 1e3 * k["ms"] / k["launches"], "gcell_s": k["updates"] / (k["ms"] / 1e3) / 1e9,
            "all_kernels_ms": {name: {"launches": v["launches"], "ms": round(v["ms"], 4)} for name, v in prof.items()}}


def _peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    return json.loads(f.read_text()) if f.exists() else {"hbm_gbs": 6800.0}


def run_mean_blur(args):
    """Mean blur: mapstencil(mean, StencilArray(rand(1000,1000), Window(1))), Float64, Remove(0.0),
    Conditional, one map per step; device time per map with L2 flushed before each."""
    import torch
    entry.build()
    st = entry.load_package()
    from stencils_gb300 import _lib
    from oracle import oracle as orc
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    rng = np.random.Generator(np.random.PCG64(1))
    a = np.asfortranarray(rng.random((1000, 1000)))
    d = st.to_device(a)
    sa = st.StencilArray(d, st.Window(1))
    out = st.mapstencil(st.mean, sa)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    _lib.profile_enable(True)
    t = _timed_steps(lambda: st.mapstencil_(st.mean, out, sa, sync=False), args.steps, args.warmup, flush)
    prof = _lib.profile_report()
    _lib.profile_enable(False)
    exact = np.array_equal(st.to_host(out).view(np.uint64),
                           orc.map(a, A.F64, st.Window(1), st.mean, st.Remove(0.0), st.Conditional()).view(np.uint64))
    thr = orc.max_threads()
    t0 = time.perf_counter()
    reps = 0
    while time.perf_counter() - t0 < 3.0:
        orc.map(a, A.F64, st.Window(1), st.mean, st.Remove(0.0), st.Conditional(), nthreads=thr)
        reps += 1
    cpu = reps * 1e6 / (time.perf_counter() - t0) / 1e9
    line = {"workload": "mean blur 1000x1000 Float64, Window(1), Remove(0), Conditional", "metric": METRIC,
            "value": args.steps * 1e6 / t / 1e9, "unit": UNIT, "us_per_map": 1e6 * t / args.steps,
            "bit_exact_vs_oracle": bool(exact), "kernel": _kernel_roofline(prof, _peaks()["hbm_gbs"]),
            "cpu_baseline": {"value": cpu, "unit": UNIT, "cores": thr, "kind": "port"},
            "reference_published": {"cpu_min_ms": 2.755, "mx330_min_ms": 0.9168, "gtx1080_ms": 0.216}}
    print(json.dumps(line), flush=True)


def _gauss_weights(st):
    import math
    w = np.array([math.exp(-d * d / (2 * 1.5 ** 2)) for d in st.Window(3).distances()])
    return w / w.sum()


def run_gauss(args):
    """7x7 Gaussian filter: Kernel(Window(3)) normalised Gaussian (sigma 1.5) on 8192^2 Float32 U[0,1), Remove(0);
    FP32 and BF16 storage; max relative error against the FP64 oracle (over the whole grid)."""
    import torch
    entry.build()
    st = entry.load_package()
    from stencils_gb300 import _lib
    from oracle import oracle as orc
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    rng = np.random.Generator(np.random.PCG64(3))
    a32 = np.asfortranarray(rng.random((8192, 8192), dtype=np.float32))
    w = _gauss_weights(st)
    ref = orc.map(np.asfortranarray(a32.astype(np.float64)), A.F64, st.Kernel(st.Window(3), w), st.kernelproduct,
                  st.Remove(0.0), st.Conditional(), nthreads=orc.max_threads())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    res = {}
    for name, tdt in (("f32", torch.float32), ("bf16", torch.bfloat16)):
        d = st.to_device(a32)
        if tdt != torch.float32:
            d2 = st.colmajor_empty(a32.shape, tdt)
            d2.copy_(d)
            d = d2
        K = st.Kernel(st.Window(3), w.astype(np.float32), weight_dtype="f32")
        sa = st.StencilArray(d, K, st.Remove(0.0))
        out = st.mapstencil(st.kernelproduct, sa)
        _lib.profile_enable(True)
        t = _timed_steps(lambda: st.mapstencil_(st.kernelproduct, out, sa, sync=False), args.steps, args.warmup, flush)
        prof = _lib.profile_report()
        _lib.profile_enable(False)
        got = out.float().cpu().numpy().T.T.astype(np.float64)
        rel = np.max(np.abs(got - ref) / np.abs(ref))
        res[name] = {"gcell_s": args.steps * a32.size / t / 1e9, "ms_per_map": 1e3 * t / args.steps,
                     "max_rel_err_vs_fp64": float(rel), "kernel": _kernel_roofline(prof, _peaks()["hbm_gbs"])}
        del d, out, sa
    line = {"workload": "7x7 Gaussian Kernel(Window(3)) 8192x8192, Remove(0)", "metric": METRIC, "unit": UNIT,
            "value": res["f32"]["gcell_s"], "results": res, "fma_bound_note": "49 FMA per cell"}
    print(json.dumps(line), flush=True)


def run_diffusion(args):
    """3D diffusion: VonNeumann(1,3) explicit diffusion c + 0.1 (sum - 6c) on 512^3 U[0,1), Wrap, 200 steps,
    FP32 and BF16 storage; FP64 total-mass drift on the GPU (K4); max relative error vs the FP64
    oracle measured on a 96^3 grid run the same 200 steps."""
    import torch
    entry.build()
    st = entry.load_package()
    from stencils_gb300 import _lib
    from oracle import oracle as orc
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    rng = np.random.Generator(np.random.PCG64(4))
    steps = 200
    side = args.side or 512
    a = np.asfortranarray(rng.random((side, side, side), dtype=np.float32))
    small = np.asfortranarray(rng.random((96, 96, 96), dtype=np.float32))
    pa, pb = np.asfortranarray(small.astype(np.float64)), np.asfortranarray(small.astype(np.float64))
    in_b = orc.map_steps(pa, pb, A.F64, st.VonNeumann(1, 3), st.Diffusion(0.1), st.Wrap(), st.Conditional(), steps,
                         nthreads=orc.max_threads())
    ref_small = pb if in_b else pa
    res = {}
    for name, tdt in (("f32", torch.float32), ("bf16", torch.bfloat16)):
        def mk(arr):
            d = st.to_device(arr)
            if tdt != torch.float32:
                d2 = st.colmajor_empty(arr.shape, tdt)
                d2.copy_(d)
                d = d2
            return d
        S = st.SwitchingStencilArray(mk(a), st.VonNeumann(1, 3), st.Wrap())
        m0 = st.mass(S.source)
        torch.cuda.synchronize()
        _lib.profile_enable(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        S = st.mapstencil_(st.Diffusion(0.1), S, steps=steps)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        prof = _lib.profile_report()
        _lib.profile_enable(False)
        m1 = st.mass(S.source)
        Ss = st.mapstencil_(st.Diffusion(0.1), st.SwitchingStencilArray(mk(small), st.VonNeumann(1, 3), st.Wrap()),
                            steps=steps)
        got = Ss.source.float().cpu().numpy().astype(np.float64)
        rel = float(np.max(np.abs(got - ref_small) / np.abs(ref_small)))
        res[name] = {"gcell_s": a.size * steps / t / 1e9, "s_total": t, "mass_drift_rel": (m1 - m0) / m0,
                     "max_rel_err_vs_fp64_96cube": rel, "kernel": _kernel_roofline(prof, _peaks()["hbm_gbs"])}
        del S, Ss
    line = {"workload": f"7-point diffusion VonNeumann(1,3) {side}^3, Wrap, 200 steps", "metric": METRIC, "unit": UNIT,
            "value": res["f32"]["gcell_s"], "results": res}
    print(json.dumps(line), flush=True)


def _batched_jobs(st, rng, n=256):
    import math
    k5 = rng.standard_normal(25).astype(np.float32)
    sten = [(st.mean, st.Window(1)), (st.mean, st.Circle(3)), (st.sum, st.Cross(2)),
            (st.kernelproduct, st.Kernel(st.Window(2), k5, weight_dtype="f32"))]
    jobs = []
    for _ in range(n):
        side = int(round(math.exp(rng.uniform(math.log(64), math.log(2048)))))
        red, hood = sten[int(rng.integers(4))]
        bnd = st.Wrap() if rng.random() < 0.5 else st.Remove(0.0)
        jobs.append((rng.random((side, side), dtype=np.float32), red, hood, bnd, int(rng.integers(1, 51))))
    return jobs


def run_batched(args):
    """Batched uneven grids: 256 Float32 grids, side log-uniform [64, 2048], stencil from {Window(1) mean, Circle(3) mean,
    Cross(2) sum, 5x5 N(0,1) kernel}, 1-50 steps, Remove or Wrap: one graph-captured persistent launch
    (autotuned) against 256 plain synchronising mapstencil! loops."""
    import torch
    entry.build()
    st = entry.load_package()
    rng = np.random.Generator(np.random.PCG64(5))
    jobs = _batched_jobs(st, rng)
    cells = sum(a.size * n for a, _, _, _, n in jobs)
    dev = [st.to_device(a) for a, *_ in jobs]

    def make():
        b = st.Batch()
        for d, (a, red, hood, bnd, n) in zip(dev, jobs):
            c = st.colmajor_empty(d.shape, d.dtype)
            c.copy_(d)
            b.add(red, st.SwitchingStencilArray(c, hood, bnd, st.Conditional()), n)
        return b
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    b = make()
    t0 = time.perf_counter()
    b.plan(autotune=True)
    plan_s = time.perf_counter() - t0
    tb = _timed_steps(lambda: b.run(sync=False), args.steps, args.warmup, flush)
    seq = make()
    seq.plan(autotune=False)
    ts = _timed_steps(seq.run_sequential, max(2, args.steps // 3), 1, flush)
    tb_s, ts_s = tb / args.steps, ts / max(2, args.steps // 3)
    line = {"workload": "256 uneven Float32 grids (Window(1) mean, Circle(3) mean, Cross(2) sum, 5x5 kernel mix)", "metric": METRIC, "unit": UNIT,
            "value": cells / tb_s / 1e9, "ms_per_batch": 1e3 * tb_s, "plain_ms": 1e3 * ts_s,
            "plain_gcell_s": cells / ts_s / 1e9, "speedup_vs_plain": ts_s / tb_s, "cell_steps": cells,
            "plan_and_autotune_s": plan_s}
    print(json.dumps(line), flush=True)


def run_serving(args):
    """Serving stream: Poisson arrivals at several rates; jobs {side log-uniform [128, 4096], Float32 / BF16 /
    UInt8, the batched-workload stencils or Moore(1) Life, steps U{1..200}}; continuous batching against the same
    arrivals served one at a time by plain calls (host->device, mapstencil! loop, device->host)."""
    import math
    import torch
    entry.build()
    st = entry.load_package()
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    from oracle.oracle import f32_to_bf16_bits
    rng = np.random.Generator(np.random.PCG64(6))
    njobs = args.serve_jobs
    k5 = rng.standard_normal(25).astype(np.float32)
    sten = [(st.mean, st.Window(1)), (st.mean, st.Circle(3)), (st.sum, st.Cross(2)),
            (st.kernelproduct, st.Kernel(st.Window(2), k5, weight_dtype="f32"))]

    def make_job():
        side = int(round(math.exp(rng.uniform(math.log(128), math.log(4096)))))
        kind = ["f32", "bf16", "u8"][int(rng.integers(3))]
        steps = int(rng.integers(1, 201))
        if kind == "u8" or rng.random() < 0.2:
            g = (rng.random((side, side)) < 0.3).astype(np.uint8)
            return g, None, st.Moore(1), st.life, st.Wrap(), steps
        red, hood = sten[int(rng.integers(4))]
        bnd = st.Wrap() if rng.random() < 0.5 else st.Remove(0.0)
        g = rng.random((side, side), dtype=np.float32)
        if kind == "bf16":
            return np.asfortranarray(f32_to_bf16_bits(g)), A.BF16, hood, (st.mean if red is st.sum else red), bnd, steps
        return np.asfortranarray(g), None, hood, red, bnd, steps

    def plain(job):
        g, code, hood, red, bnd, steps = job
        if code == A.BF16:
            t = st.colmajor_empty(g.shape, torch.bfloat16)
            t.view(torch.int16).copy_(torch.from_numpy(g.view(np.int16)))
        else:
            t = st.to_device(g)
        S = st.mapstencil_(red, st.SwitchingStencilArray(t, hood, bnd, st.Conditional()), steps=steps)
        S.source.cpu()

    rates = [float(r) for r in args.serve_rates.split(",")]
    out = {}
    for rate in rates:
        jobs = [make_job() for _ in range(njobs)]
        cells = sum(j[0].size * j[5] for j in jobs)
        gaps = rng.exponential(1.0 / rate, size=njobs)
        arrivals = np.cumsum(gaps) - gaps[0]
        # served: submit at the arrival times
        with st.Server(hbm_fraction=0.8, steps_per_tick=args.serve_tick) as srv:
            ids = []
            t0 = time.perf_counter()
            for j, at in zip(jobs, arrivals):
                dt = at - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                g, code, hood, red, bnd, steps = j
                ids.append(srv.submit(g, hood, red, bnd, steps, code=code))
            srv.drain(600.0)
            makespan = time.perf_counter() - t0
            lat = [srv.fetch(i)[1] for i in ids]
        # plain: one job at a time in arrival order (FIFO), latency = finish - arrival
        plain(jobs[0])
        torch.cuda.synchronize()
        service = []
        for j in jobs:
            t1 = time.perf_counter()
            plain(j)
            torch.cuda.synchronize()
            service.append(time.perf_counter() - t1)
        fin, plat = 0.0, []
        for at, sv in zip(arrivals, service):
            fin = max(fin, at) + sv
            plat.append(fin - at)
        out[str(int(rate))] = {
            "served": {"gcell_s": cells / makespan / 1e9, "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                       "p99_ms": 1e3 * float(np.percentile(lat, 99)), "makespan_s": makespan},
            "plain_sequential": {"gcell_s": cells / fin / 1e9, "p50_ms": 1e3 * float(np.percentile(plat, 50)),
                                 "p99_ms": 1e3 * float(np.percentile(plat, 99)), "makespan_s": fin},
            "jobs": njobs, "cell_steps": cells}
    best = max(out.values(), key=lambda v: v["served"]["gcell_s"])
    line = {"workload": "serving stream, Poisson arrivals, mixed jobs (sides 128-4096, f32/bf16/u8, 1-200 steps)", "metric": METRIC, "unit": UNIT,
            "value": best["served"]["gcell_s"], "rates": out, "steps_per_tick": args.serve_tick}
    print(json.dumps(line), flush=True)


def run_terms(args):
    """Maps over two arrays: mapstencil(f, A, B) with f = center(hood_A) + 0.1 * sum(neighbors(hood_B)) (the
    reference's diffusion-with-source form), Float64 4096x4096, Moore(1), Remove(0) on both; bit-exact
    against the oracle on the full grid; CPU baseline = the oracle on all host cores."""
    import torch
    entry.build()
    st = entry.load_package()
    from stencils_gb300 import _lib
    from oracle import oracle as orc
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    rng = np.random.Generator(np.random.PCG64(7))
    n = 4096
    a = np.asfortranarray(rng.random((n, n)))
    b = np.asfortranarray(rng.random((n, n)))
    f = st.Terms(st.center, st.scaled(0.1, st.sum))
    sa = st.StencilArray(st.to_device(a), st.Moore(1), st.Remove(0.0))
    sb = st.StencilArray(st.to_device(b), st.Moore(1), st.Remove(0.0))
    out = st.mapstencil(f, sa, sb)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    _lib.profile_enable(True)
    t = _timed_steps(lambda: st.mapstencil_(f, out, sa, sb, sync=False), args.steps, args.warmup, flush)
    prof = _lib.profile_report()
    _lib.profile_enable(False)
    items = [(a.copy(order="F"), st.Moore(1), st.Remove(0.0), st.Conditional()),
             (b.copy(order="F"), st.Moore(1), st.Remove(0.0), st.Conditional())]
    thr = orc.max_threads()
    t0 = time.perf_counter()
    want = orc.map_terms(f, items, A.F64, nthreads=thr)
    cpu_s = time.perf_counter() - t0
    exact = st.to_host(out).tobytes(order="F") == want.tobytes(order="F")
    line = {"workload": "two-array map center(A) + 0.1*sum(neighbors(B)), Float64 4096x4096, Moore(1), Remove(0)",
            "metric": METRIC, "unit": UNIT, "value": args.steps * n * n / t / 1e9, "us_per_map": 1e6 * t / args.steps,
            "bit_exact_vs_oracle": bool(exact), "kernel": _kernel_roofline(prof, _peaks()["hbm_gbs"]),
            "cpu_baseline": {"value": n * n / cpu_s / 1e9, "unit": UNIT, "cores": thr, "kind": "port",
                             "sample": "one full map"}}
    print(json.dumps(line), flush=True)


def run_scatter(args):
    """scatterstencil!(f, +, dest, source): every cell scatters its centre value to its Moore(1) neighbours, Float64
    4096x4096, Remove(0), dest accumulated in place; bit-exact against the oracle (the reference's pass
    schedule, the columns of each pass on all host threads), which is also the CPU baseline."""
    import operator
    import torch
    entry.build()
    st = entry.load_package()
    from stencils_gb300 import _lib
    from oracle import oracle as orc
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    rng = np.random.Generator(np.random.PCG64(8))
    n = 4096
    src = np.asfortranarray(rng.random((n, n)))
    sa = st.StencilArray(st.to_device(src), st.Moore(1), st.Remove(0.0))
    dest = st.to_device(np.zeros((n, n), order="F"))
    f = st.scatter_center
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    _lib.profile_enable(True)
    t = _timed_steps(lambda: st.scatterstencil_(f, operator.add, dest, sa), args.steps, args.warmup, flush)
    prof = _lib.profile_report()
    _lib.profile_enable(False)
    calls = args.warmup + args.steps
    d1 = st.to_device(np.zeros((n, n), order="F"))
    st.scatterstencil_(f, operator.add, d1, sa)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    thr = orc.max_threads()
    want = orc.scatter(f, operator.add, np.zeros((n, n), order="F"), src.copy(order="F"), A.F64, st.Moore(1),
                       st.Remove(0.0), st.Conditional(), nthreads=thr)
    cpu_s = time.perf_counter() - t0
    exact = st.to_host(d1).tobytes(order="F") == want.tobytes(order="F")
    line = {"workload": "scatterstencil! centre value to Moore(1) neighbours with +, Float64 4096x4096, Remove(0)",
            "metric": METRIC, "unit": UNIT, "value": args.steps * n * n / t / 1e9, "us_per_call": 1e6 * t / args.steps,
            "bit_exact_vs_oracle_one_call": bool(exact), "calls_accumulated": calls,
            "kernel": _kernel_roofline(prof, _peaks()["hbm_gbs"]),
            "cpu_baseline": {"value": n * n / cpu_s / 1e9, "unit": UNIT, "cores": thr, "kind": "port",
                             "sample": "one full scatter, the columns of each pass on threads as the reference's"}}
    print(json.dumps(line), flush=True)


def run_shapes(args):
    """The remaining shapes (offset-table kernel) and boundaries: one map per step on 8192^2 Float32
    U[0,1) for each (stencil, reduction, boundary, padding) below, through mapstencil_; Halo paddings
    include the ring refresh each map (update_boundary!, as the reference's gatherstencil! does).  Each
    result is compared bit for bit with the oracle on the full grid; the oracle on all host cores is the
    CPU baseline."""
    import statistics
    import torch
    entry.build()
    st = entry.load_package()
    from stencils_gb300 import _lib
    from oracle import oracle as orc
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    n = 8192
    rng = np.random.Generator(np.random.PCG64(11))
    a = np.asfortranarray(rng.random((n, n), dtype=np.float32))
    combos = [
        ("Annulus(3) mean, Remove(0), Conditional", st.Annulus(3), st.mean, st.Remove(0.0), st.Conditional()),
        ("Diamond(2) sum, Reflect, Conditional", st.Diamond(2), st.sum, st.Reflect(), st.Conditional()),
        ("Rectangle((-2,1),(-1,3)) mean, Wrap, Conditional", st.Rectangle((-2, 1), (-1, 3)), st.mean, st.Wrap(),
         st.Conditional()),
        ("Window(1) mean, Use, Halo{:in} (output 8190^2)", st.Window(1), st.mean, st.Use(), st.Halo("in")),
        ("Circle(3) mean, Reflect, Halo{:out}", st.Circle(3), st.mean, st.Reflect(), st.Halo("out")),
    ]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    thr = orc.max_threads()
    res = []
    for name, hood, red, bnd, pad in combos:
        sa = st.StencilArray(st.to_device(a), hood, bnd, pad)
        out = st.mapstencil(red, sa)
        cells = int(np.prod(out.shape))
        _lib.profile_enable(True)
        t = _timed_steps(lambda: st.mapstencil_(red, out, sa, sync=False), args.steps, args.warmup, flush)
        prof = _lib.profile_report()
        _lib.profile_enable(False)
        got = st.to_host(out)
        parent = st.to_host(sa.parent)
        t0 = time.perf_counter()
        want = orc.map(parent, A.F32, hood, red, bnd, pad, nthreads=thr)
        cpu_s = time.perf_counter() - t0
        res.append({"case": name, "taps": len(hood), "gcell_s": args.steps * cells / t / 1e9,
                    "us_per_map": 1e6 * t / args.steps, "bit_exact_vs_oracle": got.tobytes(order="F") ==
                    want.tobytes(order="F"), "kernel": _kernel_roofline(prof, _peaks()["hbm_gbs"]),
                    "cpu_gcell_s": cells / cpu_s / 1e9})
        del sa, out
    line = {"workload": "remaining shapes and boundaries, Float32 8192x8192, one map per step", "metric": METRIC,
            "unit": UNIT, "value": statistics.median(r["gcell_s"] for r in res), "value_is": "median over cases",
            "results": res, "cpu_baseline": {"unit": UNIT, "cores": thr, "kind": "port",
                                             "sample": "one full map per case (cpu_gcell_s per case)"}}
    print(json.dumps(line), flush=True)


WORKLOADS = {"mean_blur": run_mean_blur, "gauss": run_gauss, "diffusion": run_diffusion, "batched": run_batched,
             "terms": run_terms, "scatter": run_scatter, "shapes": run_shapes,
             "serving": run_serving}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="life", choices=["life"] + sorted(WORKLOADS),
                    help="life (the headline line) or one of the other benchmark workloads")
    ap.add_argument("--side", type=int, default=0, help="diffusion: grid side (default 512)")
    ap.add_argument("--serve-jobs", type=int, default=120)
    ap.add_argument("--serve-rates", default="100,300,1000,3000,5000")
    ap.add_argument("--serve-tick", type=int, default=32)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    entry.load_package()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "life":
        return WORKLOADS[args.workload](args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
