"""Writes tests/golden/seeded/: each seeded case's inputs and the oracle's output as raw column-major
binaries, and manifest.toml (shape, element type, SHA-256 per array; the case's description, the
reference call it restates and its tolerance).  Run from the repository root:

    python tests/golden/make_seeded_fixtures.py

The oracle is built first if needed (gcc).  Outputs are a few KB per case.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
OUT = HERE / "seeded"

JULIA_TYPE = {"F64": "Float64", "F32": "Float32", "BF16": "BFloat16", "U8": "UInt8"}


def code_name(abi, code):
    return next(n for n in ("F64", "F32", "BF16", "F16", "U8", "BOOL", "I32", "I64") if getattr(abi, n) == code)


def array_entry(abi, name, arr, code, fname):
    data = arr.tobytes(order="F")
    (OUT / fname).write_bytes(data)
    cn = code_name(abi, code)
    return {"file": fname, "eltype": JULIA_TYPE[cn], "abi": cn, "numpy": arr.dtype.str,
            "shape": list(arr.shape), "sha256": hashlib.sha256(data).hexdigest()}


def toml_str(x):
    return json.dumps(x)   # TOML basic strings share JSON's escapes for this ASCII text


def main():
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(HERE))
    import __graft_entry__ as entry
    st = entry.load_package()
    import stencils_gb300._abi as abi
    from oracle import oracle as orc
    import seeded_cases as S
    orc.build()
    OUT.mkdir(exist_ok=True)
    lines = ["# Seeded parity fixtures: inputs and oracle outputs as raw column-major binaries.",
             "# Written by tests/golden/make_seeded_fixtures.py; read by tests/test_seeded_fixtures.py and",
             "# run_reference.jl.  BFloat16 arrays are stored as their 16-bit patterns.", ""]
    for case in S.CASES:
        inputs = case.make_inputs(st, abi)
        out, ocode = case.run("oracle", st, abi, orc, inputs)
        lines += [f"[{case.name}]", f"description = {toml_str(case.description)}",
                  f"julia = {toml_str(case.julia)}", f"tolerance = {toml_str(case.tolerance)}", ""]
        arrays = [(k, a, c) for k, (a, c) in inputs.items()] + [("out", out, ocode)]
        for k, a, c in arrays:
            e = array_entry(abi, k, a, c, f"{case.name}.{k}.bin")
            lines.append(f"[{case.name}.arrays.{k}]")
            for key in ("file", "eltype", "abi", "numpy", "sha256"):
                lines.append(f"{key} = {toml_str(e[key])}")
            lines.append(f"shape = {json.dumps(e['shape'])}")
            lines.append("")
        print(f"{case.name}: " + ", ".join(f"{k} {a.shape} {a.dtype}" for k, a, _ in arrays))
    (OUT / "manifest.toml").write_text("\n".join(lines))


if __name__ == "__main__":
    main()
