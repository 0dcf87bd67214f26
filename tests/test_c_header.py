"""include/stencil_cuda.h is a plain C header: a C99 program that includes it, fills the descriptors and
links libstencilcuda.so builds with gcc and calls the entry points that need no device (version,
status strings, result types, an argument check that fails before any device work)."""
import shutil
import subprocess

import pytest

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "stencil_cuda.h"

int main(void) {
    int32_t offs[18];
    int k = 0;
    for (int y = -1; y <= 1; ++y)
        for (int x = -1; x <= 1; ++x) { offs[k++] = x; offs[k++] = y; }
    stc_grid src, dst;
    memset(&src, 0, sizeof src);
    memset(&dst, 0, sizeof dst);
    src.ndims = dst.ndims = 2;
    src.dtype = dst.dtype = STC_F64;
    src.size[0] = dst.size[0] = 8;
    src.size[1] = 8;
    dst.size[1] = 7;                      /* "Source array sizes must match" */
    src.stride[0] = dst.stride[0] = 1;
    src.stride[1] = dst.stride[1] = 8;
    src.data = (void*)0x10000;
    dst.data = (void*)0x20000;
    stc_stencil st;
    memset(&st, 0, sizeof st);
    st.ndims = 2;
    st.len = 9;
    st.radius = 1;
    st.offsets = offs;
    stc_op op;
    memset(&op, 0, sizeof op);
    op.code = STC_OP_MEAN;
    stc_bc bc;
    memset(&bc, 0, sizeof bc);
    bc.boundary = STC_REMOVE;
    bc.padding = STC_CONDITIONAL;
    int rc = stc_map(&src, &dst, 0, &st, &op, &bc, NULL, 0);
    printf("%d %d %s %d\n", stc_abi_version(), rc, stc_strerror(rc), stc_result_dtype(STC_OP_MEAN, STC_U8, 0));
    return 0;
}
"""


def test_header_compiles_as_c99_and_links(lib, tmp_path):
    from stencils_gb300 import _lib
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no gcc")
    import torch
    if torch.cuda.is_available():
        pytest.skip("the placeholder-address call runs only without a visible GPU")
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    so = Path(_lib.LIB_PATH)
    (tmp_path / "t.c").write_text(PROGRAM)
    exe = tmp_path / "t"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", str(root / "include"), str(tmp_path / "t.c"),
                    "-o", str(exe), str(so), f"-Wl,-rpath,{so.parent}"], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split(maxsplit=2)
    assert out[0] == "2" and out[1] == "-1"
    assert "sizes must match" in out[2]
    assert out[2].strip().endswith(" 0")      # mean of UInt8 -> Float64 (code 0)
