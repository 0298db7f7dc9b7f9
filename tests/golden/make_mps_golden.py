"""Makes tests/golden/mps_golden.npz: samaya's own MPS reader (samaya::read_mps_from_string,
reference src/io/mps_reader.cpp:517, compiled into oracle/_ref by oracle/Makefile.ref) run on
every case of mps_cases.py.

Accepted cases: the Model as arrays (A in CSC form, objective, bounds, integer flags, sense,
offset, name, row and column names). Rejected cases: whether samaya raises or reads the text, and
for a raise the line number of its message (0 for a whole-model check).

    python tests/golden/make_mps_golden.py     (needs the reference checkout)
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

KEYS = ("colptr", "rowidx", "vals", "obj", "col_lower", "col_upper", "col_integer", "row_lower",
        "row_upper", "row_starts", "col_starts")


def samaya_line(message: str) -> int:
    m = re.match(r"line (\d+): ", message)
    return int(m.group(1)) if m else 0


def main():
    from oracle import ref
    from mps_cases import accepted_cases, rejected_cases
    out = {}
    for name, text in accepted_cases():
        try:
            r = ref.mps_read_text(text)
        except ref.RefMpsError as e:
            raise SystemExit(f"samaya rejects the accepted case {name}: {e}")
        assert r["q_nnz"] == 0 and r["quadratic_rows"] == 0, name
        for k in KEYS:
            out[f"{name}__{k}"] = np.asarray(r[k])
        out[f"{name}__meta"] = np.array([r["m"], r["n"], int(r["maximize"])], dtype=np.int64)
        out[f"{name}__offset"] = np.array([r["obj_offset"]])
        for k in ("name", "row_names", "col_names"):
            out[f"{name}__{k}"] = np.frombuffer(r[k], dtype=np.uint8)
    for name, text, _, samaya in rejected_cases():
        try:
            ref.mps_read_text(text)
            got, line = "reads", 0
        except ref.RefMpsError as e:
            got, line = "raises", samaya_line(str(e))
        assert got == samaya, (name, got)
        out[f"rejected__{name}"] = np.array([1 if got == "raises" else 0, line], dtype=np.int64)
    path = os.path.join(HERE, "mps_golden.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
