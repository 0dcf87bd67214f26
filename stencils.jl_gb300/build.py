"""Compile libstencilcuda.so in-tree: every csrc/*.cu for sm_103a, in parallel, then link.

nvcc cross-compiles without a GPU; the result lands in stencils.jl_gb300/_build/ (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
OUT_DIR = PKG / "_build"
LIB = OUT_DIR / "libstencilcuda.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden", "-I", str(INCLUDE)]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(CSRC.glob("*.cu"))


def _headers():
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")))


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=(), debug: bool = False) -> Path:
    """Compile and link the library; debug=True builds libstencilcuda_debug.so (in _build/debug/) with the
    kernels' device-side bounds tests compiled in (-DSTC_DEBUG_BOUNDS)."""
    out_dir = OUT_DIR / "debug" if debug else OUT_DIR
    lib = out_dir / "libstencilcuda_debug.so" if debug else LIB
    if debug:
        extra_flags = (*extra_flags, "-DSTC_DEBUG_BOUNDS")
    out_dir.mkdir(parents=True, exist_ok=True)
    headers = _headers()
    srcs = _sources()
    objs = []
    jobs = []
    for s in srcs:
        o = out_dir / (s.stem + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra_flags, "-c", str(s), "-o", str(o)]
            jobs.append((s, cmd))
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(workers) as ex:
            futs = {ex.submit(subprocess.run, cmd, capture_output=True, text=True): s for s, cmd in jobs}
            errors = []
            for f in cf.as_completed(futs):
                r = f.result()
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout + r.stderr)
                if r.returncode != 0:
                    errors.append(f"{futs[f].name}:\n{r.stderr}")
            if errors:
                raise RuntimeError("nvcc failed:\n" + "\n".join(errors))
    if force or _stale(lib, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
    return lib


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, debug="--debug" in sys.argv))
