"""Two ways to run a reference-style mapstencil: through the CPU oracle or through the GPU library.

Both take numpy arrays in Julia axis order and return numpy results, so the same golden test
body runs against the oracle (CPU suite) and against libstencilcuda.so (GPU suite).
"""
from __future__ import annotations

import numpy as np


class OracleBackend:
    name = "oracle"

    def __init__(self, st, orc, A):
        self.st, self.orc, self.A = st, orc, A

    def _code(self, a, code=None):
        return self.A.numpy_dtype_code(a.dtype) if code is None else code

    def _parent(self, a, stencil, padding):
        st = self.st
        R = stencil.radius
        if isinstance(padding, st.Halo) and padding.kind == "out":
            p = np.zeros(tuple(s + 2 * R for s in a.shape), dtype=a.dtype, order="F")
            p[tuple(slice(R, R + s) for s in a.shape)] = a
            return p
        return np.array(a, order="F", copy=True)

    def map(self, a, stencil, red, boundary, padding, code=None):
        """mapstencil(f, StencilArray(a, stencil; boundary, padding))"""
        c = self._code(a, code)
        p = self._parent(a, stencil, padding)
        return self.orc.map(p, c, stencil, red, boundary, padding)

    def switch_map(self, a, stencil, red, boundary, padding, steps=1, code=None):
        """S = SwitchingStencilArray(a, ...); S = mapstencil!(f, S) `steps` times; the logical array of S."""
        st = self.st
        c = self._code(a, code)
        pa = self._parent(a, stencil, padding)
        pb = pa.copy(order="F")
        halo = isinstance(padding, st.Halo)
        pad = st.Halo("in") if halo else st.Conditional()
        in_b = self.orc.map_steps(pa, pb, c, stencil, red, boundary, pad, steps)
        res = pb if in_b else pa
        if halo:
            R = stencil.radius
            res = res[tuple(slice(R, s - R) for s in res.shape)]
        return np.asfortranarray(res)


class GpuBackend:
    name = "gpu"

    def __init__(self, st, A):
        self.st, self.A = st, A

    def _dev(self, a, code=None):
        import torch
        if code == self.A.BF16:
            t = torch.from_numpy(np.asfortranarray(a).astype(np.int16).view(np.int16))
            d = self.st.colmajor_empty(a.shape, torch.bfloat16)
            d.view(torch.int16).copy_(t)
            return d
        if code == self.A.BOOL:
            return self.st.to_device(a.astype(np.bool_))
        return self.st.to_device(a)

    def _host(self, t):
        import torch
        if t.dtype == torch.bfloat16:
            return np.asfortranarray(t.view(torch.int16).cpu().numpy().view(np.uint16))
        if t.dtype == torch.bool:
            return np.asfortranarray(t.cpu().numpy().astype(np.uint8))
        return self.st.to_host(t)

    def map(self, a, stencil, red, boundary, padding, code=None):
        st = self.st
        sa = st.StencilArray(self._dev(a, code), stencil, boundary, padding)
        out = st.mapstencil(red, sa)
        return self._host(out)

    def switch_map(self, a, stencil, red, boundary, padding, steps=1, code=None):
        st = self.st
        S = st.SwitchingStencilArray(self._dev(a, code), stencil, boundary, padding)
        S = st.mapstencil_(red, S, steps=steps)
        res = self._host(S.source)
        if isinstance(padding, st.Halo):
            R = stencil.radius
            res = res[tuple(slice(R, s - R) for s in res.shape)]
        return np.asfortranarray(res)
