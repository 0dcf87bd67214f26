"""The debug build (libstencilcuda_debug.so, kernels compiled with their device-side bounds tests): small
odd-sized grids through every major path report no failed test and match the oracle, and a failed test
surfaces as STC_ERR_BOUNDS on the next synchronising call of the same stream — reported, never a trap.
Runs in child processes (this process holds the release library)."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def _debug_env():
    r = subprocess.run([sys.executable, "-c", "import __graft_entry__ as e; e.load_package(); from stencils_gb300 import build; "
                        "print(build.build(debug=True))"],
                       cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    return dict(os.environ, STC_DEBUG_BOUNDS="1")


def test_debug_build_small_grids(cuda):
    env = _debug_env()
    r = subprocess.run([sys.executable, str(ROOT / "tests" / "_debug_bounds_child.py")], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert r.stdout.strip().startswith("ok")


def test_debug_build_reports_bounds_failure(cuda):
    env = _debug_env()
    code = ("import __graft_entry__ as e; st = e.load_package(); import numpy as np, torch\n"
            "from stencils_gb300 import _lib\n"
            "lib = _lib.load(); assert lib.stc_debug_bounds() == 1\n"
            "s = torch.cuda.Stream()\n"
            "with torch.cuda.stream(s):\n"
            "    assert lib.stc_debug_report_bounds(_lib.current_stream_handle()) == 0\n"
            "    S = st.SwitchingStencilArray(st.to_device(np.ones((40, 30), np.float32)), st.Window(1), st.Wrap())\n"
            "    try:\n"
            "        st.mapstencil_(st.mean, S, steps=1)\n"
            "        raise SystemExit('no error reported')\n"
            "    except _lib.StencilError as err:\n"
            "        assert err.status == -14, err.status\n"
            "    st.mapstencil_(st.mean, S, steps=1)   # read once, then clear\n"
            "print('ok')\n")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-4000:])
    assert r.stdout.strip().endswith("ok")
