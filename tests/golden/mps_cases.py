"""MPS texts for the fast reader's parity tests (tests/test_mps.py) and their golden fixture
(make_mps_golden.py): every section and rule of samaya's free-MPS reader (reference
src/io/mps_reader.cpp) that a linear model uses, the edge cases of its line handling, generated
LPs large enough to be cut into several ranges, and inputs that free MPS rejects.

Each accepted case is (name, text); each rejected case is (name, text, status, samaya) with status
the fast reader's code ("parse" or "unsupported") and samaya what samaya's reader does with it
("raises", or "reads" where it falls back to fixed MPS or reads a quadratic section).
"""
from __future__ import annotations

import os
import sys

import numpy as np

_ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

ALL_FEATURES = """NAME  features
* a comment line
OBJSENSE MAX
ROWS
 N  obj
 E  r1
 L  r2
 G  r3
 N  freerow
 E  r4
 L  r5
 G  r6
COLUMNS
 x1  obj  1.5  r1  2
 x1  r2  -3  freerow  4
 x2  r1  1  r3  5
 x2  r6  2.5
    MARKER  'MARKER'  'INTORG'
 y1  r2  1  obj  -2
 y2  r4  7
    MARKER  'MARKER'  'INTEND'
 z  r5  1  r6  -1
 z  obj  0.25
 w  r4  3
RHS
 RHS  r1  4  r2  6
 RHS  r3  1  obj  7
 r4  -2
 RHS  r5  10  r6  -3
 RHS  freerow  99
RANGES
 RNG  r1  -2  r3  4
 RNG  r4  5
 r5  2.5
 RNG  r6  -1.5
BOUNDS
 UP  BND  x1  -4
 LO  BND  x2  -1
 UP  BND  x2  3
 BV  BND  y1
 LI  BND  y2  2
 UI  BND  y2  9
 FR  BND  z
 MI  w
 UP  BND  w  8
ENDATA
junk after the end is ignored
"""

OBJSENSE_SECTION = """NAME sense
OBJSENSE
    MAXIMIZE
OBJNAME
    cost
ROWS
 N obj
 N cost
 L c1
COLUMNS
 a obj 1 cost 2
 a c1 1
 b cost -1 c1 1
RHS
 rhs c1 4 obj 3
 rhs cost 5
ENDATA
"""

OBJNAME_HEADER = """NAME objname
OBJNAME second
OBJSENSE min
ROWS
 N first
 N second
 G g1
COLUMNS
 a first 1 second 2
 a g1 1
RHS
 rhs g1 1
BOUNDS
 PL bnd a
ENDATA
"""

OBJNAME_IS_A_CONSTRAINT = """NAME objrow
OBJNAME r2
ROWS
 N n0
 E r1
 E r2
 L r3
COLUMNS
 a n0 1 r1 1
 a r2 2 r3 1
 b r1 1 r2 -1
 b r3 2
RHS
 rhs r1 1 r2 5
 rhs r3 4
BOUNDS
 UP bnd b 3
 UP bnd a 2
 LO bnd b 1
ENDATA
"""

COMMENTS_CRLF_TABS = ("NAME\tcrlf\r\n*comment\r\nROWS\r\n N\tobj\r\n\r\n E\tr1\r\n   \r\n"
                      " L r2\r\nCOLUMNS\r\n\tx\tobj\t1\tr1\t1\r\n* inside\r\n x\tr2\t2\r\n\r\n"
                      "\ty\tr1\t-1\r\nRHS\r\n rhs\tr1\t3\r\n rhs r2 4\r\nBOUNDS\r\n UP\tbnd\tx\t"
                      "10\r\n\t\r\nENDATA\r\n")

REPEATED_COLUMNS = """NAME repeats
ROWS
 N obj
 E r1
 E r2
 E r3
COLUMNS
 x1 r3 1.5 r1 2
 x2 r2 1 obj 3
 x1 r1 0.5 obj 1
 x3 r1 0 r2 -0.0
 x2 r2 -1
 x1 r2 4
RHS
 rhs r1 1
COLUMNS
 x2 r3 6 obj 0.5
 x4 r1 1 r1 2
 x1 r3 1
ENDATA
"""

INFINITIES = """NAME inf
ROWS
 N obj
 L r1
 G r2
 E r3
COLUMNS
 a obj 1 r1 1
 a r2 1 r3 1
 b r1 2 r2 -1
 c r3 1
 d r1 1
 e r2 1
RHS
 rhs r1 1e30 r2 -1e30
 rhs r3 5
BOUNDS
 UP bnd a 1e30
 LO bnd b -1e30
 UP bnd b 1e31
 LO bnd c -inf
 UP bnd c Infinity
 LO bnd d -1e29
 UP bnd d 2e29
 UP bnd e -1e20
ENDATA
"""

EMPTY_MODEL = "NAME nothing\nROWS\n N obj\nENDATA\n"

NO_NAME_NO_END = "ROWS\n N obj\n E r\nCOLUMNS\n x r 1\nRHS\n rhs r 2"

LONG_NAMES = """NAME long
ROWS
 N objective_function_with_a_long_name
 E constraint[0,1]
 E Constraint[0,1]
 L c.2_(x)
COLUMNS
 flow_from_plant_12_to_market_345 objective_function_with_a_long_name 3.25
 flow_from_plant_12_to_market_345 constraint[0,1] 1 Constraint[0,1] 2
 X1 c.2_(x) 1
 x1 c.2_(x) -1 constraint[0,1] 1
 été Constraint[0,1] 1
RHS
 rhs constraint[0,1] 1 Constraint[0,1] 2
 rhs c.2_(x) 3
ENDATA
"""

RHS_LAST_WINS = """NAME rhs
ROWS
 N obj
 E r1
 L r2
COLUMNS
 x r1 1 r2 1
RHS
 rhs r1 1
 rhs r1 2 r2 3
 rhs obj 4
 rhs obj -5
RANGES
 rng r2 1
 rng r2 -2
ENDATA
"""

BOUND_FORMS = """NAME bounds
ROWS
 N obj
 E r
COLUMNS
 x1 r 1
 x2 r 1
 x3 r 1
 x4 r 1
 x5 r 1
 x6 r 1
 x7 r 1
 BND r 1
RHS
 rhs r 1
BOUNDS
 FR x1
 FR BND x2
 MI x3 junk
 PL BND x4 5
 BV BND x5
 UP BND x6 -5
 LO BND x7 0
 UP BND x7 -5
 FR BND BND
 UP BND x1 3
 LO x2 -2
ENDATA
"""

NEGATIVE_UPPER = """NAME negup
ROWS
 N obj
 G r
COLUMNS
 a r 1
 b r 1
 c r 1
 d r 1
RHS
 rhs r -10
BOUNDS
 UP bnd a -5
 LO bnd b 0
 UP bnd b -5
 UP bnd c -5
 LO bnd c 1
 MI bnd d
 UP bnd d -1
ENDATA
"""


def _numbers_case(seed: int = 0, count: int = 400) -> str:
    """Matrix entries and bounds in many number forms (integers, decimals, exponents, '+',
    leading and trailing points, long mantissas, subnormals)."""
    rng = np.random.default_rng(seed)
    forms = []
    for k in range(count):
        v = float(rng.standard_normal() * 10.0 ** int(rng.integers(-12, 12)))
        f = k % 10
        if f == 0:
            t = repr(v)
        elif f == 1:
            t = f"{v:.3e}"
        elif f == 2:
            t = str(int(rng.integers(-10**6, 10**6)))
        elif f == 3:
            t = f"{v:.17g}"
        elif f == 4:
            t = "+" + f"{abs(v):.6f}"
        elif f == 5:
            t = f"{int(rng.integers(1, 999))}."
        elif f == 6:
            t = "." + str(int(rng.integers(1, 10**6)))
        elif f == 7:
            t = f"{v:.25e}".replace("e", "E")
        elif f == 8:
            t = "12345678901234567890123" + ("e-20" if rng.random() < 0.5 else ".5")
        else:
            t = f"{float(rng.random()) * 1e-310:.6e}"
        if float(t) == 0.0:
            t = "1"
        forms.append(t)
    lines = ["NAME numbers", "ROWS", " N obj"] + [f" E r{i}" for i in range(20)] + ["COLUMNS"]
    for k, t in enumerate(forms):
        lines.append(f" c{k // 4} r{(7 * k) % 20} {t}" if k % 4 else f" c{k // 4} obj {t}")
    lines += ["RHS"] + [f" rhs r{i} {forms[i]}" for i in range(20)]
    lines += ["BOUNDS"] + [f" UP bnd c{j} {forms[j].lstrip('+-') or '1'}" for j in range(count // 4)]
    lines.append("ENDATA")
    return "\n".join(lines) + "\n"


def _marker_case(n: int = 600) -> str:
    """Integer blocks that open and close many times (markers cut across ranges)."""
    lines = ["NAME markers", "ROWS", " N obj", " L cap", " G dem", "COLUMNS"]
    for j in range(n):
        if j % 7 == 0:
            lines.append(f"    MARKER{j} 'MARKER' '{'INTORG' if (j // 7) % 2 == 0 else 'INTEND'}'")
        lines.append(f" v{j} obj {j % 5 + 1} cap {j % 3 + 1}")
        lines.append(f" v{j} dem 1")
    lines += ["RHS", " rhs cap 100 dem 10", "ENDATA"]
    return "\n".join(lines) + "\n"


def _generated(kind: str, seed: int):
    """A generated LP written by samaya_gb300.mps.mps_lines (columns two entries to a line)."""
    from samaya_gb300 import generators as g
    from samaya_gb300.mps import mps_lines
    rng = np.random.default_rng(seed)
    if kind == "random":
        model = g.random_sparse_lp(120, 300, seed=seed)
        # every bound and row kind
        cl, cu = model.col_lower.copy(), model.col_upper.copy()
        pick = rng.integers(0, 5, model.n)
        cl[pick == 1], cu[pick == 1] = -np.inf, np.inf
        cl[pick == 2] = -np.inf
        cu[pick == 3] = np.inf
        cl[pick == 4] = cu[pick == 4] = rng.standard_normal(int((pick == 4).sum()))
        rl, ru = model.row_lower.copy(), model.row_upper.copy()
        rk = rng.integers(0, 4, model.m)
        rl[rk == 1] = -np.inf
        ru[rk == 2] = np.inf
        ru[rk == 3] = rl[rk == 3] + rng.random(int((rk == 3).sum()))
        from samaya_gb300.model import Model
        model = Model(**{**model.__dict__, "col_lower": cl, "col_upper": cu, "row_lower": rl,
                         "row_upper": ru, "maximize": bool(seed % 2), "obj_offset": 1.25})
        integer = (rng.random(model.n) < 0.2).astype(np.uint8)
    elif kind == "transport":
        model = g.transportation_lp(40, 60, seed=seed)
        integer = None
    else:
        model = g.power_law_lp(m=1000, n=2000, seed=seed)
        integer = None
    return "\n".join(mps_lines(model, name=f"{kind}{seed}", col_integer=integer)) + "\n"


def _fixed(t, a, b="", v="", c="", w=""):
    """One fixed-MPS data line: type in columns 2-3, names in 5-12, 15-22 and 40-47, values in
    25-36 and 50-61."""
    s = " " + t.ljust(2) + " " + a.ljust(8) + "  " + b.ljust(8) + "  " + v.rjust(12)
    if c:
        s += "   " + c.ljust(8) + "  " + w.rjust(12)
    return s.rstrip()


def fixed_format_case() -> str:
    """Fixed MPS with a column name that contains a space (Netlib style): free MPS rejects it,
    and it is read as fixed MPS."""
    f = _fixed
    lines = ["NAME          FIXED", "ROWS", f("N", "COST"), f("L", "LIM1"), "COLUMNS",
             f("", "MY VAR", "COST", "1.", "LIM1", "1."), f("", "X2", "COST", "2.", "LIM1", "1."),
             "RHS", f("", "RHS", "LIM1", "4."), "ENDATA"]
    return "\n".join(lines) + "\n"


def fixed_format_full_case() -> str:
    """Fixed MPS with every section: row and column names with spaces, two entries to a line,
    set names, ranges, bound types, integer markers, OBJSENSE as a section."""
    f = _fixed
    lines = ["NAME          FULL FIXED", "OBJSENSE", "    MAX", "ROWS", f("N", "PROFIT"),
             f("E", "BAL 1"), f("L", "CAP A"), f("G", "DEM B"), f("L", "R4"), "COLUMNS",
             f("", "PROD 1", "PROFIT", "3.5", "BAL 1", "1."),
             f("", "PROD 1", "CAP A", "2."),
             f("", "PROD 2", "PROFIT", "-1.25", "DEM B", "1."),
             f("", "PROD 2", "BAL 1", "-1.", "R4", "0.5"),
             f("", "MARKER", "'MARKER'", "", "'INTORG'"),
             f("", "INT X", "PROFIT", "2.", "CAP A", "1."),
             f("", "INT X", "R4", "1."),
             f("", "MARKER", "'MARKER'", "", "'INTEND'"),
             f("", "SLACK", "DEM B", "1.", "R4", "-1."),
             "RHS", f("", "RHS SET", "BAL 1", "0.", "CAP A", "10."),
             f("", "RHS SET", "DEM B", "2.", "R4", "7.5"),
             f("", "RHS SET", "PROFIT", "-4."),
             "RANGES", f("", "RNG", "BAL 1", "3."), f("", "RNG", "R4", "-2."),
             "BOUNDS", f("UP", "BND", "PROD 1", "4."), f("LO", "BND", "PROD 2", "-1."),
             f("UP", "BND", "INT X", "6."), f("MI", "BND", "SLACK"),
             f("UP", "BND", "SLACK", "-0.5"),
             "ENDATA"]
    return "\n".join(lines) + "\n"


def accepted_cases():
    cases = [("all_features", ALL_FEATURES), ("objsense_section", OBJSENSE_SECTION),
             ("objname_header", OBJNAME_HEADER),
             ("objname_is_a_constraint", OBJNAME_IS_A_CONSTRAINT),
             ("comments_crlf_tabs", COMMENTS_CRLF_TABS),
             ("repeated_columns", REPEATED_COLUMNS), ("infinities", INFINITIES),
             ("empty_model", EMPTY_MODEL), ("no_name_no_end", NO_NAME_NO_END),
             ("long_names", LONG_NAMES), ("rhs_last_wins", RHS_LAST_WINS),
             ("bound_forms", BOUND_FORMS), ("negative_upper", NEGATIVE_UPPER),
             ("numbers", _numbers_case()), ("markers", _marker_case()),
             ("fixed_format", fixed_format_case()), ("fixed_format_full", fixed_format_full_case())]
    for kind, seeds in (("random", (1, 2)), ("transport", (3,)), ("powerlaw", (4,))):
        for seed in seeds:
            cases.append((f"{kind}_{seed}", _generated(kind, seed)))
    return cases


_BASE = """NAME bad
ROWS
 N obj
 E r1
 L r2
COLUMNS
 x obj 1 r1 1
 x r2 2
 y r1 1
RHS
 rhs r1 1
BOUNDS
 UP bnd x 4
ENDATA
"""


def _edit(old: str, new: str) -> str:
    assert old in _BASE
    return _BASE.replace(old, new, 1)


def rejected_cases():
    return [
        ("unknown_row", _edit(" y r1 1", " y r9 1"), "parse", "raises"),
        ("bad_number", _edit(" y r1 1", " y r1 1.2.3"), "parse", "raises"),
        ("number_out_of_range", _edit(" y r1 1", " y r1 1e400"), "parse", "raises"),
        ("exponent_without_digits", _edit(" y r1 1", " y r1 1e"), "parse", "raises"),
        ("double_plus", _edit(" y r1 1", " y r1 ++1"), "parse", "raises"),
        ("four_fields", _edit(" y r1 1", " y r1 1 r2"), "parse", "raises"),
        ("duplicate_row", _edit(" L r2", " L r2\n E r1"), "parse", "raises"),
        ("unknown_row_type", _edit(" L r2", " X r2"), "parse", "raises"),
        ("duplicate_before_bad_row", _edit(" L r2", " L r2\n E r1\n G r3\n X r4"), "parse",
         "raises"),
        ("row_without_name", _edit(" L r2", " L"), "parse", "raises"),
        ("unknown_section", _edit("RHS\n", "FOO\nRHS\n"), "parse", "raises"),
        ("data_before_section", " x y\n" + _BASE, "parse", "raises"),
        ("data_after_name", _edit("NAME bad\n", "NAME bad\n stray line\n"), "parse", "raises"),
        ("objname_after_rows", _edit("COLUMNS\n", "OBJNAME r1\nCOLUMNS\n"), "parse", "raises"),
        ("range_on_objective", _edit("BOUNDS\n", "RANGES\n rng obj 1\nBOUNDS\n"), "parse",
         "raises"),
        ("rhs_field_count", _edit(" rhs r1 1", " rhs r1 1 r2"), "parse", "raises"),
        ("bound_unknown_column", _edit(" UP bnd x 4", " UP bnd q 4"), "parse", "raises"),
        ("bound_unknown_type", _edit(" UP bnd x 4", " XX bnd x 4"), "parse", "raises"),
        ("bound_semicontinuous", _edit(" UP bnd x 4", " SC bnd x 4"), "parse", "raises"),
        ("bound_too_short", _edit(" UP bnd x 4", " UP"), "parse", "raises"),
        ("bound_missing_value", _edit(" UP bnd x 4", " UP x"), "parse", "raises"),
        ("bound_five_fields", _edit(" UP bnd x 4", " FR bnd x 4 5"), "parse", "raises"),
        ("unknown_marker", _edit(" y r1 1", "    M 'MARKER' 'INTXX'\n y r1 1"), "parse",
         "raises"),
        ("sos_section", _edit("ENDATA", "SOS\n S1 set\nENDATA"), "parse", "raises"),
        ("infinite_entry", _edit(" y r1 1", " y r1 1e30"), "parse", "raises"),
        ("infinite_offset", _edit(" rhs r1 1", " rhs r1 1 obj 1e30"), "parse", "raises"),
        ("lower_plus_infinity", _edit(" UP bnd x 4", " LO bnd x 1e30"), "parse", "raises"),
        ("nan_bound", _edit(" UP bnd x 4", " UP bnd x nan"), "parse", "raises"),
        ("empty_text", "", "parse", "raises"),
        ("name_only", "NAME x\nENDATA\n", "parse", "raises"),
        ("unknown_sense", _edit("ROWS\n", "OBJSENSE\n    UP\nROWS\n"), "parse", "raises"),
        ("columns_before_rows", "NAME x\nCOLUMNS\n x r 1\nROWS\n N obj\n E r\nENDATA\n",
         "parse", "raises"),
        ("quadobj", _edit("ENDATA", "QUADOBJ\n x x 2\n x y 1\nENDATA"), "unsupported",
         "reads"),
        ("qmatrix", _edit("ENDATA", "QMATRIX\n x x 2\nENDATA"), "unsupported", "reads"),
        ("qcmatrix", _edit("ENDATA", "QCMATRIX r2\n x x 1\nENDATA"), "unsupported", "reads"),
    ]
