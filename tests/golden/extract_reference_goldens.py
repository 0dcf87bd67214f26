"""Extract the golden vectors of Stencils.jl's own test suite into reference_goldens.json.

Run where a Stencils.jl checkout is available (it reads the Julia test files as text; nothing is
executed):  python tests/golden/extract_reference_goldens.py /path/to/Stencils.jl
(or set STENCILS_JL_DIR to that path).

Each entry records the reference file and line range it came from.  Matrix literals are
parsed from Julia syntax (`[a b; c d]` or rows on separate lines) into row-major nested lists,
so entry[i][j] is the Julia element [i+1, j+1].  The parity tests read only the JSON.
"""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path


# (name, file, first line, last line, kind)  kind: matrix | vector | tuples
ENTRIES = [
    # test/array.jl — the hot path
    ("indices_remove_moore_4x4_at_1_1", "test/array.jl", 7, 7, "tuples"),
    ("indices_wrap_moore_4x4_at_1_1", "test/array.jl", 9, 9, "tuples"),
    ("indices_reflect_moore_4x4_at_1_1", "test/array.jl", 11, 11, "tuples"),
    ("indices_switching_reflect_moore_4x4_at_1_1", "test/array.jl", 13, 13, "tuples"),
    ("mean_remove_window1_5x6", "test/array.jl", 139, 145, "matrix"),
    ("sum_use_halo_in_window1_5x6_interior", "test/array.jl", 157, 161, "matrix"),
    ("mean_wrap_window1_1d", "test/array.jl", 181, 181, "vector"),
    ("mean_wrap_halo_in_window1_1d", "test/array.jl", 182, 182, "vector"),
    ("mean_wrap_window1_5x6", "test/array.jl", 200, 206, "matrix"),
    ("mean_reflect_window1_1d", "test/array.jl", 228, 228, "vector"),
    ("mean_reflect_halo_in_window1_1d", "test/array.jl", 229, 229, "vector"),
    ("mean_reflect_window1_5x6", "test/array.jl", 247, 253, "matrix"),
    # test/stencils.jl — shapes, neighbours, kernels, named stencils
    ("init_6x6", "test/stencils.jl", 3, 8, "matrix"),
    ("offsets_moore_1_2", "test/stencils.jl", 28, 28, "tuples"),
    ("offsets_window_1_2", "test/stencils.jl", 48, 49, "tuples"),
    ("offsets_vonneumann_1_2", "test/stencils.jl", 63, 63, "tuples"),
    ("neighbors_vonneumann_init_at_2_2", "test/stencils.jl", 70, 70, "vector"),
    ("offsets_vonneumann_2_2", "test/stencils.jl", 74, 76, "tuples"),
    ("offsets_annulus_1", "test/stencils.jl", 83, 84, "tuples"),
    ("neighbors_annulus_init_at_2_2", "test/stencils.jl", 91, 91, "vector"),
    ("offsets_annulus_2", "test/stencils.jl", 95, 96, "tuples"),
    ("offsets_ordinal_1", "test/stencils.jl", 103, 103, "tuples"),
    ("neighbors_ordinal_init_at_2_2", "test/stencils.jl", 110, 110, "vector"),
    ("offsets_ordinal_2", "test/stencils.jl", 114, 114, "tuples"),
    ("offsets_cardinal_1", "test/stencils.jl", 121, 121, "tuples"),
    ("neighbors_cardinal_init_at_2_2", "test/stencils.jl", 128, 128, "vector"),
    ("offsets_cardinal_2", "test/stencils.jl", 132, 132, "tuples"),
    ("win_5x5", "test/stencils.jl", 136, 140, "matrix"),
    ("positional_h1_offsets", "test/stencils.jl", 141, 141, "tuples"),
    ("neighbors_positional_h1_win_at_3_3", "test/stencils.jl", 146, 146, "vector"),
    ("positional_h2_offsets", "test/stencils.jl", 150, 150, "tuples"),
    ("neighbors_positional_h2_win_at_3_3", "test/stencils.jl", 154, 154, "vector"),
    ("rectangle_A_5x5", "test/stencils.jl", 160, 164, "matrix"),
    ("neighbors_rectangle_h1_at_3_3", "test/stencils.jl", 172, 172, "vector"),
    ("neighbors_rectangle_h3_3d_at_2_2_1", "test/stencils.jl", 182, 182, "vector"),
    ("named_n_w_center_minus_win", "test/stencils.jl", 207, 213, "matrix"),
    ("named_cardinal_W_plus_S", "test/stencils.jl", 222, 228, "matrix"),
    ("named_ordinal_NE_plus_NW", "test/stencils.jl", 233, 239, "matrix"),
    ("kernel_positional_offsets", "test/stencils.jl", 298, 298, "tuples"),
]

NUM = r"-?\d+(?:\.\d+)?(?:e-?\d+)?"


def _lines(ref: Path, rel: str, a: int, b: int) -> str:
    text = (ref / rel).read_text().splitlines()
    return "\n".join(text[a - 1: b])


def parse_tuples(src: str):
    # every innermost (a, b[, c]) tuple of integers, in order, right of a comparison if any
    if "==" in src:
        src = src[src.rindex("==") + 2:]
    return [[int(x) for x in re.findall(r"-?\d+", t)]
            for t in re.findall(r"\((\s*-?\s*\d+\s*(?:,\s*-?\s*\d+\s*)+)\)", src.replace("- ", "-"))]


def parse_vector(src: str):
    # the last [...] or SVector(...) literal on the line
    m = re.findall(r"(?:SVector)?[\[(]([^\[\]()]*)[\])]", src)
    body = m[-1]
    return [float(x) for x in re.findall(NUM, body)]


def parse_matrix(src: str):
    end = src.rindex("]")
    body = src[src.rindex("[", 0, end) + 1: end]
    rows = []
    for chunk in re.split(r"[;\n]", body):
        vals = re.findall(NUM, chunk)
        if vals:
            rows.append([float(v) for v in vals])
    width = len(rows[0])
    assert all(len(r) == width for r in rows), f"ragged matrix literal: {src!r}"
    return rows


def main(ref_dir: str | None = None):
    ref_dir = ref_dir or os.environ.get("STENCILS_JL_DIR")
    if not ref_dir:
        raise SystemExit("usage: extract_reference_goldens.py /path/to/Stencils.jl (or set STENCILS_JL_DIR)")
    ref = Path(ref_dir)
    out = {"source": "Stencils.jl test suite (test/array.jl, test/stencils.jl), extracted as text",
           "entries": {}}
    for name, rel, a, b, kind in ENTRIES:
        src = _lines(ref, rel, a, b)
        data = {"matrix": parse_matrix, "vector": parse_vector, "tuples": parse_tuples}[kind](src)
        out["entries"][name] = {"where": f"{rel}:{a}-{b}", "kind": kind, "data": data}
    path = Path(__file__).with_name("reference_goldens.json")
    path.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {path} ({len(ENTRIES)} entries)")


if __name__ == "__main__":
    main(*sys.argv[1:])
