"""Benchmark of the mapstencil hot path on GB300 (one JSON line on rank 0).

Headline workload (one "step"): Conway's Life on a 4096x4096 UInt8 grid, initial density 0.3
Bernoulli from seed 2, Moore(1) B3/S23, Wrap boundary, Halo padding, SwitchingStencilArray: 1000
generations of `A = mapstencil!(life, A)`.  Inputs are synthetic (seeded numpy PCG64).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload NAME]

`value`      whole-job Gcell-updates/s with the state resident in HBM (device-timed, CUDA events,
             L2 flushed between timed steps by writing a 256 MiB buffer).
`e2e`        the same metric through the public API with pinned host buffers: every step copies the
             initial grid host->device into the Halo parent's interior (one pitched copy), runs the
             1000 generations, and copies the result back (one pitched copy).
`roofline`   the dominant kernel's algorithmic bytes (1 B read + 1 B written per cell update) per
             launch over its CUDA-event launch time, against the HBM copy bandwidth; `issue_frac` is
             the same launch against the integer-issue ceiling its measured instruction count allows.
`cpu_baseline` the oracle (a C restatement of the reference's gather, OpenMP; for Moore(1) Life on
             UInt8 Halo parents the specialised loop the reference's compiled kernel amounts to) on
             the host cores, on a bounded number of generations of the same grid.
`configs`    the other benchmark configurations (mean blur 1000^2 Float64; 7x7 Gaussian 8192^2 in
             Float32 / BFloat16 / Float16 storage; 512^3 diffusion x 200 in the same three; 256 batched
             uneven grids; the serving stream at five arrival rates), each with its own clock record,
             end-to-end figure, relative error against FP64 where it applies, and a roofline against
             the unit that binds it.  `--workload NAME` prints one of them alone.
--impl reference times the headline's CPU implementation as the reference arm (rank 0 only).
N > 1 runs N independent replicas (the path has no data exchange between GPUs).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import queue
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
SMSP_PER_SM = 4


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
            return self
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()
        return self

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


def _peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    p = json.loads(f.read_text()) if f.exists() else {}
    return {"hbm_gbs": float(p.get("hbm_gbs", 6800.0)), "source": "measured" if "hbm_gbs" in p else "fallback"}


def _traffic():
    f = ROOT / "profiles" / "traffic.json"
    return json.loads(f.read_text()) if f.exists() else {}


def _device_facts():
    import torch
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    return {"sms": props.multi_processor_count}


def _clock_hz(clk: dict) -> float:
    return (clk.get("sm_mhz") or clk.get("sm_max_mhz") or 2070.0) * 1e6


def _issue_frac(updates_per_s: float, warp_inst_per_update: float, clk: dict) -> dict:
    """Fraction of the instruction-issue ceiling: every SM sub-partition issues at most one warp
    instruction per clock, so updates/s <= SMs x 4 x clock / (warp instructions per update)."""
    sms = _device_facts()["sms"]
    ceiling = sms * SMSP_PER_SM * _clock_hz(clk) / warp_inst_per_update
    return {"issue_ceiling_gcell_s": ceiling / 1e9, "issue_frac": updates_per_s / ceiling,
            "warp_inst_per_update": warp_inst_per_update}


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


# ------------------------------------------------------------------ GPU arm: the headline
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

    # e2e through the public API with pinned host buffers and one pitched copy each way
    pinned_in = torch.empty(SIDE * SIDE, dtype=torch.uint8).pin_memory()
    pinned_in.copy_(torch.from_numpy(np.asfortranarray(a0).ravel(order="F")))
    pinned_out = torch.empty(SIDE * SIDE, dtype=torch.uint8).pin_memory()
    S2 = st.SwitchingStencilArray(st.to_device(a0, dev), st.Moore(1), st.Wrap(), st.Halo("out"))
    e2e_times = []
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        barrier()
        t0 = time.perf_counter()
        # host -> the source parent's interior, 1000 generations, result interior -> host: queued in
        # stream order, the step ends when the result is in pinned host memory
        st.copy_to_device_(S2.source[1:-1, 1:-1], pinned_in, sync=False)
        S2 = st.mapstencil_(st.life, S2, steps=GENERATIONS, sync=False)
        st.copy_to_host_(pinned_out, S2.source[1:-1, 1:-1], sync=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_times.append(dt)
    # the clock record spans the three timed passes (device-timed, per-launch-traced, end to end)
    clk = clocks.stop()
    e2e_s = max_over_ranks(sum(e2e_times), dev)
    e2e_value = ws * args.steps * updates_per_step / e2e_s / 1e9

    # roofline of the dominant kernel
    peaks = _peaks()
    dom = max(prof.items(), key=lambda kv: kv[1]["ms"]) if prof else (None, None)
    roof = None
    launches = sum(v["launches"] for v in prof.values())
    if dom[0]:
        k = dom[1]
        achieved = k["alg_bytes"] / (k["ms"] / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": dom[0], "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"], "traffic": None,
                "launches": k["launches"], "avg_launch_us": 1e3 * k["ms"] / k["launches"],
                "alg_bytes_per_launch": k["alg_bytes"] / k["launches"],
                "updates_per_launch": k["updates"] / k["launches"],
                "share_of_device_time": k["ms"] / max(1e-9, sum(v["ms"] for v in prof.values())),
                "note": "effective figure: the persistent kernel keeps the packed state in shared memory for all "
                        "1000 generations, so the physical DRAM traffic (`traffic`) is far below the algorithmic "
                        "bytes; the binding unit is integer issue (issue_frac)"}
        t = _traffic().get(dom[0])
        if t:
            roof["traffic"] = t["bytes_per_launch"]
            roof["traffic_source"] = t["source"]
            if "warp_inst_per_launch" in t:
                rate = k["updates"] / (k["ms"] / 1e3)
                roof.update(_issue_frac(rate, t["warp_inst_per_launch"] / (k["updates"] / k["launches"]), clk))
                roof["issue_source"] = t["inst_source"]

    configs = None
    if not args.no_configs and rank == 0:
        configs = run_configs(args, local)
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
    if configs is not None:
        line["configs"] = configs
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ the other configurations
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


def _wall_steps(fn, steps, warmup):
    """Host-clock seconds of `steps` synchronising calls of fn() (end to end, copies included)."""
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        fn()
    torch.cuda.synchronize()
    return time.perf_counter() - t0


def _kernels(prof):
    return {name: {"launches": v["launches"], "ms": round(v["ms"], 4)} for name, v in prof.items()}


def _hbm_roof(prof, peaks):
    """Dominant kernel: algorithmic bytes per launch over its CUDA-event time, against HBM."""
    name, k = max(prof.items(), key=lambda kv: kv[1]["ms"])
    ach = k["alg_bytes"] / (k["ms"] / 1e3) / 1e9
    return name, k, {"bound": "hbm", "kernel": name, "achieved": ach, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / peaks["hbm_gbs"], "peak_source": peaks["source"],
                     "avg_launch_us": 1e3 * k["ms"] / k["launches"],
                     "kernel_gcell_s": k["updates"] / (k["ms"] / 1e3) / 1e9}


def _with_clocks(fn, args, local):
    clk = ClockSampler(local).start()
    clk.wait_first(3.0)
    t0 = time.perf_counter()
    try:
        res = fn(args)
    except Exception as exc:  # a configuration that fails is reported, the others still run
        res = {"error": f"{type(exc).__name__}: {exc}"}
    res["clocks"] = clk.stop()
    res["wall_s"] = time.perf_counter() - t0
    return res


def cfg_mean_blur(args):
    """Mean blur: mapstencil(mean, StencilArray(rand(1000,1000), Window(1))), Float64, Remove(0.0),
    Conditional, one map per step (configuration 1; the reference publishes numbers for it)."""
    import torch
    st = entry.load_package()
    from stencils_gb300 import _lib
    rng = np.random.Generator(np.random.PCG64(1))
    a = np.asfortranarray(rng.random((1000, 1000)))
    sa = st.StencilArray(st.to_device(a), st.Window(1))
    out = st.mapstencil(st.mean, sa)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    steps = max(args.steps, 50)
    _lib.profile_enable(True)
    t = _timed_steps(lambda: st.mapstencil_(st.mean, out, sa, sync=False), steps, args.warmup, flush)
    prof = _lib.profile_report()
    _lib.profile_enable(False)
    # e2e: host input (pinned) copied in, the map, the result copied back, every call
    te = _e2e_map(st, a, sa.parent, out, lambda: st.mapstencil_(st.mean, out, sa, sync=False), steps, args.warmup)
    cpu = _cpu_rate(lambda orc, A, thr: orc.map(a, A.F64, st.Window(1), st.mean, st.Remove(0.0), st.Conditional(),
                                                 nthreads=thr), 1e6, 3.0)
    name, k, roof = _hbm_roof(prof, _peaks())
    # binding unit: the FP64 pipe.  Each cell is 8 Float64 adds (the division by 9 is integer arithmetic);
    # GB300's nominal FP64 rate is 1.25 TFLOP/s counting an FMA as two, i.e. 0.625e12 FP64 instructions/s.
    fp64_ceiling = 0.625e12 / 8
    kr = k["updates"] / (k["ms"] / 1e3)
    roof.update({"binding": "fp64", "fp64_ceiling_gcell_s": fp64_ceiling / 1e9, "fp64_frac": kr / fp64_ceiling,
                 "fp64_formula": "0.625e12 FP64 instr/s (1.25 TFLOP/s nominal, FMA = 2) / 8 DADD per cell"})
    return {"workload": "mean blur 1000x1000 Float64, Window(1), Remove(0), Conditional, one map", "unit": UNIT,
            "value": steps * 1e6 / t / 1e9, "us_per_map": 1e6 * t / steps,
            "e2e": {"value": steps * 1e6 / te / 1e9, "unit": UNIT, "us_per_call": 1e6 * te / steps,
                    "h2d_bytes_per_step": 8e6, "d2h_bytes_per_step": 8e6},
            "roofline": roof, "kernels": _kernels(prof), "cpu_baseline": cpu,
            "reference_published": {"cpu_min_ms": 2.755, "cpu_gcell_s": 0.363, "mx330_min_ms": 0.9168,
                                    "gtx1080_ms": 0.216, "gtx1080_gcell_s": 4.63,
                                    "source": "Stencils.jl README (8-core ThinkPad T14; MX330; GTX 1080)"}}


def _pinned(a: np.ndarray):
    """A pinned host tensor holding a's bytes in column-major order."""
    import torch
    t = torch.empty(a.nbytes, dtype=torch.uint8).pin_memory()
    t.copy_(torch.from_numpy(np.frombuffer(np.asfortranarray(a).tobytes(order="F"), dtype=np.uint8)))
    return t


def _e2e_map(st, host_in, dev_in, dev_out, run, steps, warmup):
    """Host-clock seconds of `steps` calls of: pinned host -> dev_in (one pitched copy), run(), dev_out ->
    pinned host, each call waiting for its result on the host."""
    import torch
    pin_in = _pinned(host_in)
    pin_out = torch.empty(dev_out.numel() * dev_out.element_size(), dtype=torch.uint8).pin_memory()

    def call():
        st.copy_to_device_(dev_in, pin_in, sync=False)
        run()
        st.copy_to_host_(pin_out, dev_out, sync=False)
        torch.cuda.synchronize()
    return _wall_steps(call, steps, warmup)


def _cpu_rate(call, cells, target_s):
    """The oracle (the CPU baseline leg) on all host cores: cells per call over repeated calls."""
    from oracle import oracle as orc
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    thr = orc.max_threads()
    t0 = time.perf_counter()
    reps = 0
    while reps == 0 or time.perf_counter() - t0 < target_s:
        call(orc, A, thr)
        reps += 1
    return {"value": reps * cells / (time.perf_counter() - t0) / 1e9, "unit": UNIT, "cores": thr, "kind": "port",
            "sample": f"{reps} calls"}


def _gauss_weights(st):
    w = np.array([math.exp(-d * d / (2 * 1.5 ** 2)) for d in st.Window(3).distances()])
    return w / w.sum()


def _max_rel(got, ref) -> float:
    import torch
    return float(((got.to(torch.float64) - ref).abs() / ref.abs()).max())


def _cast(t, dtype):
    st = entry.load_package()
    out = st.colmajor_empty(tuple(t.shape), dtype, t.device)
    out.copy_(t)
    return out


def cfg_gauss(args):
    """7x7 Gaussian filter: Kernel(Window(3)) normalised Gaussian (sigma 1.5) on 8192^2 U[0,1), Remove(0);
    Float32, BFloat16 and Float16 storage with Float32 accumulation; max relative error against the
    library's Float64 path (bit-exact with the oracle)."""
    import torch
    st = entry.load_package()
    from stencils_gb300 import _lib
    rng = np.random.Generator(np.random.PCG64(3))
    a32 = np.asfortranarray(rng.random((8192, 8192), dtype=np.float32))
    w = _gauss_weights(st)
    d32 = st.to_device(a32)
    ref = st.mapstencil(st.kernelproduct, st.StencilArray(_cast(d32, torch.float64), st.Kernel(st.Window(3), w),
                                                          st.Remove(0.0)))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    K = st.Kernel(st.Window(3), w.astype(np.float32), weight_dtype="f32")
    sms = _device_facts()["sms"]
    res = {}
    for name, tdt in (("f32", torch.float32), ("bf16", torch.bfloat16), ("f16", torch.float16)):
        x = d32 if tdt == torch.float32 else _cast(d32, tdt)
        sa = st.StencilArray(x, K, st.Remove(0.0))
        out = st.mapstencil(st.kernelproduct, sa)
        _lib.profile_enable(True)
        t = _timed_steps(lambda: st.mapstencil_(st.kernelproduct, out, sa, sync=False), args.steps, args.warmup, flush)
        prof = _lib.profile_report()
        _lib.profile_enable(False)
        kname, k, roof = _hbm_roof(prof, _peaks())
        kr = k["updates"] / (k["ms"] / 1e3)
        res[name] = {"value": args.steps * a32.size / t / 1e9, "ms_per_map": 1e3 * t / args.steps,
                     "max_rel_err_vs_fp64": _max_rel(out, ref), "roofline": roof, "kernel_rate": kr}
        del x, sa, out
    # e2e (Float32): host grid in, the map, host result out through the public API
    sa32 = st.StencilArray(d32, K, st.Remove(0.0))
    out32 = st.mapstencil(st.kernelproduct, sa32)
    te = _e2e_map(st, a32, d32, out32, lambda: st.mapstencil_(st.kernelproduct, out32, sa32, sync=False), 3, 3)
    clk_hz = 2.07e9
    for r in res.values():
        # binding unit: the FP32 FMA pipe, 49 FMAs per cell (128 per SM per clock)
        ceiling = sms * 128 * clk_hz / 49
        r["roofline"].update({"binding": "fp32_fma", "fma_ceiling_gcell_s": ceiling / 1e9,
                              "fma_frac": r.pop("kernel_rate") / ceiling,
                              "fma_formula": "SMs x 128 FMA/clk x 2.07 GHz / 49 FMA per cell"})
    cpu = _cpu_rate(lambda orc, A, thr: orc.map(np.asfortranarray(a32[:1024, :1024]), A.F32, K, st.kernelproduct,
                                                 st.Remove(0.0), st.Conditional(), nthreads=thr), 1024 * 1024, 2.0)
    cpu["sample"] = "1024x1024 corner of the grid, " + cpu["sample"]
    return {"workload": "7x7 Gaussian Kernel(Window(3)) sigma 1.5, 8192x8192, Remove(0), one map", "unit": UNIT,
            "value": res["f32"]["value"], "results": res,
            "e2e": {"value": 3 * a32.size / te / 1e9, "unit": UNIT, "dtype": "f32",
                    "h2d_bytes_per_step": a32.nbytes, "d2h_bytes_per_step": a32.nbytes},
            "precision_limits": {"f32": 1e-6, "bf16": 1e-2, "f16": 1e-2}, "cpu_baseline": cpu}


def cfg_diffusion(args):
    """3D diffusion: VonNeumann(1,3), c + 0.1 (sum - 6c), 512^3 U[0,1), Wrap, 200 steps.  Float32 state
    (temporally blocked path), BFloat16 and Float16 state in the precision mode (STC_KEEP_F32) and, for
    comparison, BFloat16 rounded to nearest every step; max relative error against the library's Float64
    run of the same 200 steps, and the FP64 total-mass drift (K4)."""
    import torch
    st = entry.load_package()
    from stencils_gb300 import _lib
    rng = np.random.Generator(np.random.PCG64(4))
    steps = 200
    side = args.side or 512
    a = np.asfortranarray(rng.random((side, side, side), dtype=np.float32))
    d32 = st.to_device(a)
    cells = a.size

    def run(x, keep):
        S = st.SwitchingStencilArray(x, st.VonNeumann(1, 3), st.Wrap())
        return st.mapstencil_(st.Diffusion(0.1), S, steps=steps, keep_f32=keep)

    ref = run(_cast(d32, torch.float64), False).source
    traffic = _traffic()
    res = {}
    for name, tdt, keep in (("f32", torch.float32, False), ("bf16_keep_f32", torch.bfloat16, True),
                            ("f16_keep_f32", torch.float16, True), ("bf16_per_step", torch.bfloat16, False)):
        x = _cast(d32, tdt)
        S = st.SwitchingStencilArray(x, st.VonNeumann(1, 3), st.Wrap())
        m0 = st.mass(S.source)
        run(_cast(d32, tdt), keep)      # warm-up: workspace, kernel attributes
        torch.cuda.synchronize()
        _lib.profile_enable(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        S = st.mapstencil_(st.Diffusion(0.1), S, steps=steps, keep_f32=keep)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        prof = _lib.profile_report()
        _lib.profile_enable(False)
        m1 = st.mass(S.source)
        kname, k, roof = _hbm_roof(prof, _peaks())
        roof["note"] = "algorithmic bytes: one read and one write of the state per cell-step"
        e = traffic.get(f"{kname}:{name}")
        if e:
            # the instruction count and DRAM bytes per cell update of an ncu capture of this kernel
            roof.update(_issue_frac(k["updates"] / (k["ms"] / 1e3), e["warp_inst_per_update"], {}))
            roof["traffic_bytes_per_update"] = e["dram_bytes_per_update"]
            roof["counters_source"] = e["source"]
        res[name] = {"value": cells * steps / t / 1e9, "s_total": t, "mass_drift_rel": (m1 - m0) / m0,
                     "max_rel_err_vs_fp64": _max_rel(S.source, ref), "roofline": roof, "kernels": _kernels(prof)}
        del x, S
    del ref
    # e2e (Float32): host grid in, 200 steps, host grid out through the public API
    Se = st.SwitchingStencilArray(_cast(d32, torch.float32), st.VonNeumann(1, 3), st.Wrap())
    holder = {"S": Se}

    def run_e2e():
        holder["S"] = st.mapstencil_(st.Diffusion(0.1), holder["S"], steps=steps, sync=False)
    # steps is even, so the result lands in the parent the input went into
    te = _e2e_map(st, a, Se.source, Se.source, run_e2e, 1, 1)
    cpu = _cpu_rate(lambda orc, A, thr: orc.map_steps(np.asfortranarray(a[:128, :128, :128]),
                                                      np.asfortranarray(a[:128, :128, :128]), A.F32,
                                                      st.VonNeumann(1, 3), st.Diffusion(0.1), st.Wrap(),
                                                      st.Conditional(), 4, nthreads=thr), 128 ** 3 * 4, 2.0)
    cpu["sample"] = "4 steps of a 128^3 grid per call, " + cpu["sample"]
    return {"workload": f"7-point diffusion VonNeumann(1,3) {side}^3, Wrap, {steps} steps", "unit": UNIT,
            "value": res["f32"]["value"], "results": res,
            "e2e": {"value": cells * steps / te / 1e9, "unit": UNIT, "dtype": "f32",
                    "h2d_bytes_per_step": a.nbytes, "d2h_bytes_per_step": a.nbytes},
            "precision_limits": {"f32": 1e-6, "bf16_keep_f32": 1e-2, "f16_keep_f32": 1e-2},
            "reference_per_step_gcell_s_before_blocking": 505, "cpu_baseline": cpu}


def cfg_blocked2d(args):
    """2D multi-step maps on Float32 state: Window(1) mean and VonNeumann(1) diffusion, 8192^2 U[0,1), Wrap,
    100 steps, temporally blocked (8 steps per pass over HBM) against the per-step map (STC_TBLOCK=0)."""
    import torch
    st = entry.load_package()
    from stencils_gb300 import _lib
    rng = np.random.Generator(np.random.PCG64(6))
    steps, side = 100, (args.side or 8192)
    a = np.asfortranarray(rng.random((side, side), dtype=np.float32))
    d = st.to_device(a)
    cells = a.size
    res = {}
    for name, hood, red in (("window_mean", st.Window(1), st.mean), ("vn_diffusion", st.VonNeumann(1), st.Diffusion(0.1))):
        for mode in ("blocked", "per_step"):
            if mode == "per_step":
                os.environ["STC_TBLOCK"] = "0"
            try:
                S = st.SwitchingStencilArray(d.clone(), hood, st.Wrap())
                st.mapstencil_(red, S, steps=8)      # warm-up: kernel attributes
                torch.cuda.synchronize()
                _lib.profile_enable(True)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                S = st.mapstencil_(red, S, steps=steps)
                e1.record()
                e1.synchronize()
                t = e0.elapsed_time(e1) / 1e3
                prof = _lib.profile_report()
                _lib.profile_enable(False)
            finally:
                os.environ.pop("STC_TBLOCK", None)
            kname, k, roof = _hbm_roof(prof, _peaks())
            roof["note"] = ("algorithmic bytes: one Float32 read and one write per cell-step (a blocked pass "
                            "moves them once per 8 steps, so its effective fraction can exceed 1)")
            e = _traffic().get(f"{kname}:{name}")
            if e:
                # the binding unit: instruction issue, from an ncu capture of this kernel
                roof.update(_issue_frac(k["updates"] / (k["ms"] / 1e3), e["warp_inst_per_update"], {}))
                roof["traffic_bytes_per_update"] = e["dram_bytes_per_update"]
                roof["counters_source"] = e["source"]
            res[f"{name}_{mode}"] = {"value": cells * steps / t / 1e9, "s_total": t, "roofline": roof,
                                     "kernels": _kernels(prof)}
            del S
    for name in ("window_mean", "vn_diffusion"):
        res[f"{name}_speedup"] = res[f"{name}_blocked"]["value"] / res[f"{name}_per_step"]["value"]
    # e2e: host grid in, 100 blocked steps, host grid out
    Se = st.SwitchingStencilArray(d.clone(), st.Window(1), st.Wrap())
    holder = {"S": Se}

    def run_e2e():
        holder["S"] = st.mapstencil_(st.mean, holder["S"], steps=steps, sync=False)
    te = _e2e_map(st, a, Se.source, Se.source, run_e2e, 1, 1)   # steps even: the result is in the input parent
    cpu = _cpu_rate(lambda orc, A, thr: orc.map_steps(np.asfortranarray(a[:512, :512]), np.asfortranarray(a[:512, :512]),
                                                      A.F32, st.Window(1), st.mean, st.Wrap(), st.Conditional(), 4,
                                                      nthreads=thr), 512 * 512 * 4, 2.0)
    cpu["sample"] = "4 steps of a 512^2 grid per call, " + cpu["sample"]
    return {"workload": f"Window(1) mean and VonNeumann(1) diffusion, Float32 {side}^2, Wrap, {steps} steps",
            "unit": UNIT, "value": res["window_mean_blocked"]["value"], "results": res,
            "e2e": {"value": cells * steps / te / 1e9, "unit": UNIT, "dtype": "f32",
                    "h2d_bytes_per_step": a.nbytes, "d2h_bytes_per_step": a.nbytes},
            "cpu_baseline": cpu}


def _batched_jobs(st, rng, n=256):
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


def cfg_batched(args):
    """Batched uneven grids: 256 Float32 grids, side log-uniform [64, 2048], stencil from {Window(1) mean,
    Circle(3) mean, Cross(2) sum, 5x5 N(0,1) kernel}, 1-50 steps, Remove or Wrap: one graph-captured
    persistent launch (autotuned) against 256 plain synchronising mapstencil! loops."""
    import torch
    st = entry.load_package()
    from stencils_gb300 import _lib
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
    _lib.profile_enable(True)
    tb = _timed_steps(lambda: b.run(sync=False), args.steps, args.warmup, flush)
    prof = _lib.profile_report()
    _lib.profile_enable(False)
    seq = make()
    seq.plan(autotune=False)
    nseq = max(2, args.steps // 3)
    ts = _timed_steps(seq.run_sequential, nseq, 1, flush)
    tb_s, ts_s = tb / args.steps, ts / nseq
    # e2e: every grid copied in from host memory, the batch run, every result copied back
    host = [np.asfortranarray(a) for a, *_ in jobs]

    def e2e():
        for d, h in zip(dev, host):
            st.copy_to_device_(d, h, sync=False)
        b.run(sync=False)
        for i, h in enumerate(host):
            st.copy_to_host_(h, b.result(i).source, sync=False)
    te = _wall_steps(e2e, 3, 1) / 3
    nbytes = sum(h.nbytes for h in host)
    name, k, roof = _hbm_roof(prof, _peaks())
    return {"workload": "256 uneven Float32 grids (Window(1) mean, Circle(3) mean, Cross(2) sum, 5x5 kernel mix)",
            "unit": UNIT, "value": cells / tb_s / 1e9, "ms_per_batch": 1e3 * tb_s, "plain_ms": 1e3 * ts_s,
            "plain_gcell_s": cells / ts_s / 1e9, "speedup_vs_plain": ts_s / tb_s, "cell_steps": cells,
            "plan_and_autotune_s": plan_s, "roofline": roof, "kernels": _kernels(prof),
            "e2e": {"value": cells / te / 1e9, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes}}


def cfg_serving(args):
    """Serving stream: Poisson arrivals at each rate; jobs {side log-uniform [128, 4096], Float32 / BFloat16 /
    UInt8, the batched-workload stencils or Moore(1) Life, steps U{1..200}}.  The served arm submits each job
    at its arrival time to the continuous-batching server and fetches results as they finish; the plain arm
    runs the same arrivals concurrently against one worker that serves them first come first served, each
    as plain calls (host->device, mapstencil! loop, device->host).  Latency = result on host - arrival."""
    import torch
    st = entry.load_package()
    A = __import__("stencils_gb300._abi", fromlist=["x"])
    rng = np.random.Generator(np.random.PCG64(6))
    njobs = args.serve_jobs
    k5 = rng.standard_normal(25).astype(np.float32)
    sten = [(st.mean, st.Window(1)), (st.mean, st.Circle(3)), (st.sum, st.Cross(2)),
            (st.kernelproduct, st.Kernel(st.Window(2), k5, weight_dtype="f32"))]
    # inputs are corners of shared random pools (copied per job when submitted), so 1000 jobs need no
    # 1000 separate host arrays
    pool_f = np.asfortranarray(rng.random((4096, 4096), dtype=np.float32))
    pool_b = np.asfortranarray((pool_f.view(np.uint32) >> 16).astype(np.uint16))
    pool_u = np.asfortranarray((pool_f < 0.3).astype(np.uint8))

    def make_job():
        side = int(round(math.exp(rng.uniform(math.log(128), math.log(4096)))))
        kind = ["f32", "bf16", "u8"][int(rng.integers(3))]
        steps = int(rng.integers(1, 201))
        if kind == "u8" or rng.random() < 0.2:
            return pool_u[:side, :side], None, st.Moore(1), st.life, st.Wrap(), steps
        red, hood = sten[int(rng.integers(4))]
        bnd = st.Wrap() if rng.random() < 0.5 else st.Remove(0.0)
        if kind == "bf16":
            return pool_b[:side, :side], A.BF16, hood, (st.mean if red is st.sum else red), bnd, steps
        return pool_f[:side, :side], None, hood, red, bnd, steps

    def plain(job):
        g, code, hood, red, bnd, steps = job
        g = np.asfortranarray(g)
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
        # served
        lat = {}
        with st.Server(hbm_fraction=0.8, steps_per_tick=args.serve_tick) as srv:
            pending = {}
            t0 = time.perf_counter()
            def collect(wait_s):
                # the server's completion queue: only finished jobs are touched
                for i in srv.ready(timeout_s=wait_s):
                    srv.fetch(i)
                    lat[i] = time.perf_counter() - t0 - pending.pop(i)
            for j, at in zip(jobs, arrivals):
                while True:
                    now = time.perf_counter() - t0
                    if now >= at:
                        break
                    collect(min(0.0005, at - now))
                g, code, hood, red, bnd, steps = j
                pending[srv.submit(g, hood, red, bnd, steps, code=code)] = at
            while pending:
                collect(0.002)
            makespan = time.perf_counter() - t0
        served = np.array(list(lat.values()))
        # plain: one worker serves the arrivals in order, concurrently with their arrival
        plain(jobs[0])
        torch.cuda.synchronize()
        q = queue.Queue()
        plat = []

        def worker():
            while True:
                item = q.get()
                if item is None:
                    return
                job, at = item
                plain(job)
                plat.append(time.perf_counter() - t1 - at)
        th = threading.Thread(target=worker)
        t1 = time.perf_counter()
        th.start()
        for j, at in zip(jobs, arrivals):
            dt = at - (time.perf_counter() - t1)
            if dt > 0:
                time.sleep(dt)
            q.put((j, at))
        q.put(None)
        th.join()
        pmake = time.perf_counter() - t1
        plat = np.array(plat)
        out[str(int(rate))] = {
            "served": {"gcell_s": cells / makespan / 1e9, "p50_ms": 1e3 * float(np.percentile(served, 50)),
                       "p99_ms": 1e3 * float(np.percentile(served, 99)), "makespan_s": makespan},
            "plain": {"gcell_s": cells / pmake / 1e9, "p50_ms": 1e3 * float(np.percentile(plat, 50)),
                      "p99_ms": 1e3 * float(np.percentile(plat, 99)), "makespan_s": pmake},
            "throughput_ratio": (cells / makespan) / (cells / pmake), "jobs": njobs, "cell_steps": cells}
    return {"workload": "serving stream, Poisson arrivals, mixed jobs (sides 128-4096, f32/bf16/u8, 1-200 steps)",
            "unit": UNIT, "value": max(v["served"]["gcell_s"] for v in out.values()), "value_is": "best rate",
            "rates": out, "steps_per_tick": args.serve_tick, "jobs_per_rate": njobs,
            "e2e": {"note": "every figure of this configuration is end to end: host input to host result"}}


CONFIGS = {"mean_blur": cfg_mean_blur, "gauss": cfg_gauss, "diffusion": cfg_diffusion, "blocked2d": cfg_blocked2d,
           "batched": cfg_batched, "serving": cfg_serving}


def run_configs(args, local):
    import torch
    out = {}
    for name, fn in CONFIGS.items():
        out[name] = _with_clocks(fn, args, local)
        torch.cuda.empty_cache()
    return out


# ------------------------------------------------------------------ single extra workloads
def run_terms(args):
    """Maps over two arrays: mapstencil(f, A, B) with f = center(hood_A) + 0.1 * sum(neighbors(hood_B)) (the
    reference's diffusion-with-source form), Float64 4096x4096, Moore(1), Remove(0) on both."""
    import torch
    st = entry.load_package()
    from stencils_gb300 import _lib
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
    cpu = _cpu_rate(lambda orc, A, thr: orc.map_terms(f, items, A.F64, nthreads=thr), n * n, 1.0)
    name, k, roof = _hbm_roof(prof, _peaks())
    return {"workload": "two-array map center(A) + 0.1*sum(neighbors(B)), Float64 4096x4096, Moore(1), Remove(0)",
            "unit": UNIT, "value": args.steps * n * n / t / 1e9, "us_per_map": 1e6 * t / args.steps,
            "roofline": roof, "cpu_baseline": cpu}


def run_scatter(args):
    """scatterstencil!(f, +, dest, source): every cell scatters its centre value to its Moore(1) neighbours, Float64
    4096x4096, Remove(0), dest accumulated in place."""
    import operator
    import torch
    st = entry.load_package()
    from stencils_gb300 import _lib
    rng = np.random.Generator(np.random.PCG64(8))
    n = 4096
    src = np.asfortranarray(rng.random((n, n)))
    sa = st.StencilArray(st.to_device(src), st.Moore(1), st.Remove(0.0))
    dest = st.to_device(np.zeros((n, n), order="F"))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    _lib.profile_enable(True)
    t = _timed_steps(lambda: st.scatterstencil_(st.scatter_center, operator.add, dest, sa), args.steps, args.warmup,
                     flush)
    prof = _lib.profile_report()
    _lib.profile_enable(False)
    cpu = _cpu_rate(lambda orc, A, thr: orc.scatter(st.scatter_center, operator.add, np.zeros((n, n), order="F"),
                                                     src.copy(order="F"), A.F64, st.Moore(1), st.Remove(0.0),
                                                     st.Conditional(), nthreads=thr), n * n, 1.0)
    name, k, roof = _hbm_roof(prof, _peaks())
    return {"workload": "scatterstencil! centre value to Moore(1) neighbours with +, Float64 4096x4096, Remove(0)",
            "unit": UNIT, "value": args.steps * n * n / t / 1e9, "us_per_call": 1e6 * t / args.steps,
            "roofline": roof, "cpu_baseline": cpu}


def run_shapes(args):
    """The remaining shapes (offset-table kernel) and boundaries: one map per step on 8192^2 Float32 U[0,1) for
    each (stencil, reduction, boundary, padding) below, through mapstencil_."""
    import torch
    st = entry.load_package()
    from stencils_gb300 import _lib
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
    res = []
    for name, hood, red, bnd, pad in combos:
        sa = st.StencilArray(st.to_device(a), hood, bnd, pad)
        out = st.mapstencil(red, sa)
        cells = int(np.prod(out.shape))
        _lib.profile_enable(True)
        t = _timed_steps(lambda: st.mapstencil_(red, out, sa, sync=False), args.steps, args.warmup, flush)
        prof = _lib.profile_report()
        _lib.profile_enable(False)
        kname, k, roof = _hbm_roof(prof, _peaks())
        res.append({"case": name, "taps": len(hood), "gcell_s": args.steps * cells / t / 1e9,
                    "us_per_map": 1e6 * t / args.steps, "roofline": roof})
        del sa, out
    return {"workload": "remaining shapes and boundaries, Float32 8192x8192, one map per step", "unit": UNIT,
            "value": statistics.median(r["gcell_s"] for r in res), "value_is": "median over cases", "results": res}


WORKLOADS = dict(CONFIGS, terms=run_terms, scatter=run_scatter, shapes=run_shapes)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true", help="the headline line only")
    ap.add_argument("--workload", default="life", choices=["life"] + sorted(WORKLOADS),
                    help="life (the headline line, with every configuration under `configs`) or one configuration")
    ap.add_argument("--side", type=int, default=0, help="diffusion: grid side (default 512); blocked2d: grid side (default 8192)")
    ap.add_argument("--serve-jobs", type=int, default=1000)
    ap.add_argument("--serve-rates", default="100,300,1000,3000,5000")
    ap.add_argument("--serve-tick", type=int, default=32)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    entry.load_package()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "life":
        import torch
        entry.build()
        from stencils_gb300 import _lib
        _lib.load()
        local = dist_env()[2]
        torch.cuda.set_device(local)
        res = _with_clocks(WORKLOADS[args.workload], args, local)
        res["metric"] = METRIC
        print(json.dumps(res), flush=True)
        return 0
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
