"""Seeded random MPS texts through the fast reader and samaya's own reader (CPU test; it runs
where the samaya checkout is present): every text either reads to the same Model in both, bit
for bit, at several thread counts, or is refused by both. Where samaya raises, the fast reader
refuses at the same line. The texts mix every section, bound and row type,
markers, set names, comments, blank and CRLF lines, repeated columns and sections, number
forms and, at random, one of a set of errors."""
from __future__ import annotations

import os
import re
import sys

import numpy as np
import pytest

from samaya_gb300 import mps

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from test_mps import _assert_same, _fast_dict  # noqa: E402

ROW_TYPES = ("E", "L", "G", "N", "e", "l")
BOUND_TYPES = ("UP", "LO", "FX", "FR", "MI", "PL", "BV", "LI", "UI", "up", "Lo")


def _number(rng) -> str:
    k = int(rng.integers(0, 9))
    v = float(rng.standard_normal() * 10.0 ** int(rng.integers(-4, 5)))
    if k == 0:
        return repr(v)
    if k == 1:
        return f"{v:.4e}"
    if k == 2:
        return str(int(rng.integers(-50, 50)))
    if k == 3:
        return f"+{abs(v):.3f}"
    if k == 4:
        return f"{int(rng.integers(1, 99))}."
    if k == 5:
        return f".{int(rng.integers(1, 999))}"
    if k == 6:
        return "0" if rng.random() < 0.3 else "-7.25"
    if k == 7:
        return f"{v:.6E}"
    return f"{v:.17g}"


def _text(seed: int) -> str:
    rng = np.random.default_rng(seed)
    m = int(rng.integers(1, 12))
    n = int(rng.integers(1, 25))
    rows = [f"r{i}" for i in range(m)]
    cols = [f"c{j}" for j in range(n)] + (["r0"] if rng.random() < 0.2 else [])
    out = [f"NAME fuzz{seed}"]
    if rng.random() < 0.3:
        out.append("OBJSENSE " + ("MAX" if rng.random() < 0.5 else "minimize"))
    if rng.random() < 0.2:
        out += ["OBJNAME", f"    {('obj', 'r1', 'cost')[int(rng.integers(0, 3))]}"]
    out += ["ROWS", " N obj"]
    kinds = {}
    for r in rows:
        t = ROW_TYPES[int(rng.integers(0, len(ROW_TYPES)))]
        kinds[r] = t
        out.append(f" {t} {r}")
    if rng.random() < 0.3:
        out.append("* a comment")
    out.append("COLUMNS")
    targets = rows + ["obj"]
    pairs = {}
    in_int = False
    order = list(range(len(cols)))
    if rng.random() < 0.3:  # a column named again later, not next to its first lines
        order.append(int(rng.integers(0, len(cols))))
    for j in order:
        c = cols[j]
        if rng.random() < 0.15:
            in_int = not in_int
            out.append(f"    M{j} 'MARKER' '{'INTORG' if in_int else 'INTEND'}'")
        for _ in range(int(rng.integers(1, 4))):
            k = int(rng.integers(1, 3))
            ents = []
            for _ in range(k):
                r = targets[int(rng.integers(0, len(targets)))]
                if pairs.get((c, r), 0) >= 2:  # at most two entries per (row, column)
                    continue
                pairs[(c, r)] = pairs.get((c, r), 0) + 1
                ents.append(f"{r} {_number(rng) if rng.random() < 0.8 else '1'}")
            if ents:
                sep = "\t" if rng.random() < 0.2 else " "
                out.append(sep + c + sep + sep.join(ents))
            if rng.random() < 0.1:
                out.append("")
    if in_int and rng.random() < 0.5:
        out.append("    MEND 'MARKER' 'INTEND'")
    out.append("RHS")
    for r in rows + ["obj"]:
        if rng.random() < 0.6:
            v = _number(rng)
            if r != "obj" and rng.random() < 0.05:  # an infinite side of an L or G row
                v = {"L": "1e30", "G": "-1e30"}.get(kinds[r].upper(), v)
            out.append(f" {'rhs ' if rng.random() < 0.7 else ''}{r} {v}")
    if rng.random() < 0.4:
        out.append("RANGES")
        for r in rows:
            if rng.random() < 0.4 and kinds[r].upper() != "N":
                out.append(f" rng {r} {_number(rng)}")
    if rng.random() < 0.8:
        out.append("BOUNDS")
        for _ in range(int(rng.integers(0, 2 * len(cols) + 1))):
            t = BOUND_TYPES[int(rng.integers(0, len(BOUND_TYPES)))]
            c = cols[int(rng.integers(0, len(cols)))]
            needs = t.upper() not in ("FR", "MI", "PL", "BV")
            setname = "bnd " if rng.random() < 0.7 else ""
            v = _number(rng)
            if rng.random() < 0.05:  # infinite bounds on their own side
                v = {"UP": "1e31", "LO": "-inf"}.get(t.upper(), v)
            out.append(f" {t} {setname}{c}" + (f" {v}" if needs else ""))
    if rng.random() < 0.1:  # a second COLUMNS section adding to old and new columns
        out += ["COLUMNS", f" {cols[0]} {rows[0]} 2", " extra obj 1"]
    out.append("ENDATA")
    if rng.random() < 0.25:
        out = _break(out, rng)
    nl = "\r\n" if rng.random() < 0.15 else "\n"
    return nl.join(out) + nl


ERRORS = (
    lambda s: s.replace(" r0 ", " nosuchrow ", 1),
    lambda s: s.replace("COLUMNS", "COLUMN", 1),
    lambda s: s.replace(" E ", " X ", 1),
    lambda s: s + " stray data after the end",
    lambda s: s.replace("ROWS", "ROWS\n N obj", 1),
    lambda s: s.replace(" 1\n", " 1.2.3\n", 1),
    lambda s: s.replace(" UP bnd ", " SC bnd ", 1),
    lambda s: s.replace("'INTORG'", "'INTXX'", 1),
    lambda s: s.replace("RHS", "QUADOBJ\n c0 c0 1\nRHS", 1),
    lambda s: s.replace(" c1 ", " c1 r0 ", 1),
    lambda s: " leading data line\n" + s,
)


def _break(lines, rng):
    s = "\n".join(lines)
    return ERRORS[int(rng.integers(0, len(ERRORS)))](s).split("\n")


def _line(message: str) -> int:
    m = re.match(r"line (\d+): ", message)
    return int(m.group(1)) if m else 0


@pytest.mark.parametrize("block", range(4))
def test_random_texts_read_alike(block):
    from oracle import ref
    if not ref.available():
        pytest.skip("the samaya checkout is not present")
    ref.build()
    read = refused = 0
    for seed in range(block * 150, (block + 1) * 150):
        text = _text(seed)
        try:
            want = ref.mps_read_text(text)
        except ref.RefMpsError as e:
            want, why = None, str(e)
        for threads in (1, 3, 7):
            try:
                got = _fast_dict(mps.read_mps_text(text, threads=threads))
            except mps.MpsReadError as e:
                assert want is None or e.code == mps.SG_ERR_UNSUPPORTED, (seed, str(e))
                if want is None and e.code == mps.SG_ERR_PARSE:
                    assert _line(str(e)) == _line(why), (seed, str(e), why)
                continue
            assert want is not None, (seed, why)
            _assert_same(got, want, f"seed {seed} threads {threads}")
        if want is None:
            refused += 1
        else:
            read += 1
    assert read > 30 and refused > 10, (read, refused)


def _mutated(seed: int) -> bytes:
    """A random text with one to three byte edits: a byte replaced, a byte inserted (CR, NUL,
    blanks, newline, sign, point, exponent, quote, high bytes), a run deleted, the text cut, or
    a slice of it repeated elsewhere."""
    rng = np.random.default_rng(10_000 + seed)
    b = bytearray(_text(seed).encode())
    junk = (b"\r", b"\x00", b" ", b"\t", b"\n", b"*", b"+", b"-", b"e", b".", b"\xff",
            b"\xc3\xa9", b"'", b"1")
    for _ in range(int(rng.integers(1, 4))):
        op = int(rng.integers(0, 5))
        i = int(rng.integers(0, max(1, len(b))))
        if op == 0 and b:
            b[i] = int(rng.integers(0, 256))
        elif op == 1:
            b[i:i] = junk[int(rng.integers(0, len(junk)))]
        elif op == 2 and b:
            del b[i:i + int(rng.integers(1, 8))]
        elif op == 3:
            b = b[:i]
        else:
            j = int(rng.integers(0, max(1, len(b))))
            b[i:i] = b[j:j + int(rng.integers(1, 40))]
    return bytes(b)


def test_mutated_texts_read_alike():
    """Byte-level mutations of the random texts: the same Model or the same refusal (line) as
    samaya's reader, at 1 and 4 threads."""
    from oracle import ref
    if not ref.available():
        pytest.skip("the samaya checkout is not present")
    ref.build()
    for seed in range(400):
        text = _mutated(seed)
        try:
            want = ref.mps_read_text(text)
        except ref.RefMpsError as e:
            want, why = None, str(e)
        for threads in (1, 4):
            try:
                got = _fast_dict(mps.read_mps_text(text, threads=threads))
            except mps.MpsReadError as e:
                assert want is None or e.code == mps.SG_ERR_UNSUPPORTED, (seed, str(e))
                if want is None and e.code == mps.SG_ERR_PARSE:
                    assert _line(str(e)) == _line(why), (seed, str(e), why)
                continue
            assert want is not None, (seed, why)
            _assert_same(got, want, f"mutated seed {seed} threads {threads}")



def _fixed_text(seed: int) -> str:
    """A random fixed-MPS text: row and column names with spaces, one or two entries to a
    line, set names, ranges, bound types, markers, values of up to 12 characters; now and then
    a field out of place or an unknown name."""
    from mps_cases import _fixed as f
    rng = np.random.default_rng(20_000 + seed)
    m, n = int(rng.integers(1, 8)), int(rng.integers(1, 12))
    rows = [f"R {i}" for i in range(m)]
    cols = [f"X {j}" if j % 2 else f"COL{j}" for j in range(n)]
    kinds = ["E", "L", "G", "N"]

    def val():
        return f"{float(rng.standard_normal() * 10.0 ** int(rng.integers(-2, 3))):.6g}"[:12]
    out = ["NAME          FIX" + str(seed)]
    if rng.random() < 0.3:
        out += ["OBJSENSE", "    MAX"]
    out += ["ROWS", f("N", "OBJ")]
    rk = {}
    for r in rows:
        rk[r] = kinds[int(rng.integers(0, 4))]
        out.append(f(rk[r], r))
    out.append("COLUMNS")
    in_int = False
    for c in cols:
        if rng.random() < 0.2:
            in_int = not in_int
            out.append(f("", "MARKER", "'MARKER'", "", "'INTORG'" if in_int else "'INTEND'"))
        targets = list(rng.permutation(rows + ["OBJ"]))[:int(rng.integers(1, 4))]
        for k in range(0, len(targets), 2):
            pair = targets[k:k + 2]
            out.append(f("", c, pair[0], val(), *((pair[1], val()) if len(pair) > 1 else ())))
    if in_int:
        out.append(f("", "MARKER", "'MARKER'", "", "'INTEND'"))
    out.append("RHS")
    for r in rows + ["OBJ"]:
        if rng.random() < 0.6:
            out.append(f("", "RHS", r, val()))
    if rng.random() < 0.5:
        out.append("RANGES")
        out += [f("", "RNG", r, val()) for r in rows if rk[r] != "N" and rng.random() < 0.4]
    out.append("BOUNDS")
    for c in cols:
        t = ("UP", "LO", "FX", "MI", "PL", "BV", "FR")[int(rng.integers(0, 7))]
        out.append(f(t, "BND", c, "" if t in ("MI", "PL", "BV", "FR") else val()))
    out.append("ENDATA")
    if rng.random() < 0.2:
        i = int(rng.integers(1, len(out) - 1))
        out[i] = out[i].replace("R 0", "R 9").replace("COL0", "COLX")
    return "\n".join(out) + "\n"


def test_fixed_format_texts_read_alike():
    """Random fixed-MPS texts: the fast reader reads them as samaya's reader does (free MPS
    first, then fixed), the same Model or the same refusal, at 1 and 4 threads."""
    from oracle import ref
    if not ref.available():
        pytest.skip("the samaya checkout is not present")
    ref.build()
    read = 0
    for seed in range(200):
        text = _fixed_text(seed)
        try:
            want = ref.mps_read_text(text)
        except ref.RefMpsError as e:
            want, why = None, str(e)
        for threads in (1, 4):
            try:
                got = _fast_dict(mps.read_mps_text(text, threads=threads))
            except mps.MpsReadError as e:
                assert want is None, (seed, str(e))
                assert _line(str(e)) == _line(why), (seed, str(e), why)
                continue
            assert want is not None, (seed, why)
            _assert_same(got, want, f"fixed seed {seed} threads {threads}")
        read += want is not None
    assert read > 100, read
