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
`cpu_baseline` the oracle (a C restatement of the reference's gather, OpenMP) on the host cores, on
             a bounded number of generations of the same grid.
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
    # calibrate a bounded sample: generations per step so that one step takes about 3 s
    _, threads, _, _ = cpu_life_rate(0.5)
    rate1, _, gens, _ = cpu_life_rate(3.0, threads)
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
    sample = f"{gens} generations of the 4096x4096 grid per step, OpenMP {threads} threads"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": CONFIG,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "CPU restatement of the reference's gather (oracle/stencil_oracle.c); the reference is "
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
        S = st.mapstencil_(st.life, S, steps=GENERATIONS)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    _lib.profile_enable(True)
    evs = []
    t_wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        S = st.mapstencil_(st.life, S, steps=GENERATIONS)
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall0
    prof = _lib.profile_report()
    _lib.profile_enable(False)
    clk = clocks.stop()
    barrier()
    dev_s = sum(a.elapsed_time(b) for a, b in evs) / 1e3
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
        # source parent interior <- host (column-major grid == row-major transpose)
        S2.source[1:-1, 1:-1].T.copy_(pinned_in, non_blocking=True)
        S2 = st.mapstencil_(st.life, S2, steps=GENERATIONS)
        pinned_out.copy_(S2.source[1:-1, 1:-1].T, non_blocking=True)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            e2e_times.append(dt)
    e2e_s = max_over_ranks(sum(e2e_times), dev)
    e2e_value = ws * args.steps * updates_per_step / e2e_s / 1e9

    if rank != 0:
        return 0
    cpu = None
    if not args.no_cpu_baseline:
        rate, threads, gens, dt = cpu_life_rate(args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{gens} generations of the 4096x4096 grid ({dt:.1f} s), oracle OpenMP {threads} threads"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": CONFIG,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": SIDE * SIDE,
                    "d2h_bytes_per_step": SIDE * SIDE},
            "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": clk,
            "kernels": prof, "wall_s_timed_region": wall}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    entry.load_package()
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
