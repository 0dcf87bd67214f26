"""The committed seeded fixtures (tests/golden/seeded/, written by tests/golden/make_seeded_fixtures.py):
the oracle reproduces every output bit for bit from the committed inputs (CPU suite), the seeded
generators still produce those inputs, and the GPU library reproduces every output from the same input
files, bit for bit or within the stated kernelproduct tolerance (GPU suite)."""
import hashlib
import sys
import tomllib
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"
SEEDED = GOLDEN / "seeded"
sys.path.insert(0, str(GOLDEN))
import seeded_cases as S  # noqa: E402

MANIFEST = tomllib.loads((SEEDED / "manifest.toml").read_text())


def load_arrays(abi, name):
    out = {}
    for k, e in MANIFEST[name]["arrays"].items():
        data = (SEEDED / e["file"]).read_bytes()
        assert hashlib.sha256(data).hexdigest() == e["sha256"], f"{e['file']} changed"
        a = np.frombuffer(data, dtype=np.dtype(e["numpy"])).reshape(e["shape"], order="F")
        out[k] = (np.asfortranarray(a.copy()), getattr(abi, e["abi"]))
    return out


def test_manifest_lists_every_case():
    assert sorted(MANIFEST) == sorted(c.name for c in S.CASES)


@pytest.mark.parametrize("case", S.CASES, ids=lambda c: c.name)
def test_seeded_inputs_regenerate(case, st, abi):
    """The seeded generators still give the committed inputs (PCG64 streams, shapes, dtypes)."""
    files = load_arrays(abi, case.name)
    for k, (a, code) in case.make_inputs(st, abi).items():
        fa, fcode = files[k]
        assert code == fcode and a.shape == fa.shape and a.tobytes(order="F") == fa.tobytes(order="F"), k


@pytest.mark.parametrize("case", S.CASES, ids=lambda c: c.name)
def test_oracle_reproduces_fixture(case, st, abi, orc):
    arrays = load_arrays(abi, case.name)
    want, wcode = arrays.pop("out")
    got, gcode = case.run("oracle", st, abi, orc, arrays)
    assert gcode == wcode and got.shape == want.shape
    assert got.tobytes(order="F") == want.tobytes(order="F")


def _kdot_tolerance(st, abi, orc, arrays, want, wcode):
    """2 L 2^-24 sum|w v| through the oracle (absolute weights and values), plus one rounding of the
    stored BFloat16 result."""
    from oracle.oracle import bf16_bits_to_f32
    a, code = arrays["A"]
    w, _ = arrays["weights"]
    av = bf16_bits_to_f32(a) if code == abi.BF16 else a
    absk = st.Kernel(st.Window(3), np.abs(w).astype(np.float32), weight_dtype="f32")
    mag = orc.map(np.asfortranarray(np.abs(av).astype(np.float32)), abi.F32, absk, st.kernelproduct,
                  st.Remove(0.0), st.Conditional()).astype(np.float64)
    tol = 2 * len(w) * 2.0 ** -24 * mag + 1e-30
    wf = bf16_bits_to_f32(want).astype(np.float64) if wcode == abi.BF16 else want.astype(np.float64)
    if wcode == abi.BF16:
        tol = tol + np.abs(wf) * 2.0 ** -7 + 1e-6
    return tol, wf


@pytest.mark.gpu
@pytest.mark.parametrize("case", S.CASES, ids=lambda c: c.name)
def test_gpu_reproduces_fixture(case, cuda, st, abi, orc):
    import torch
    from oracle.oracle import bf16_bits_to_f32
    arrays = load_arrays(abi, case.name)
    want, wcode = arrays.pop("out")
    got, gcode = case.run("gpu", st, abi, orc, arrays)
    torch.cuda.synchronize()
    assert gcode == wcode and got.shape == want.shape
    if case.tolerance == "bit-exact":
        assert got.tobytes(order="F") == want.tobytes(order="F")
        return
    tol, wf = _kdot_tolerance(st, abi, orc, arrays, want, wcode)
    gf = bf16_bits_to_f32(got).astype(np.float64) if gcode == abi.BF16 else got.astype(np.float64)
    err = np.abs(gf - wf)
    assert (err <= tol).all(), f"max excess {np.max(err - tol)}"
