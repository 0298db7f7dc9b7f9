"""MPS files for the PDLP path: the engine library's fast reader (include/sg_mps.h) and a
free-MPS writer.

``read_mps`` reads an MPS file (free MPS, and fixed MPS where free fails) on several host
threads into the arrays of samaya::Model, the model samaya::read_mps (reference
src/io/mps_reader.cpp:530-541) builds from it. What the fast reader declines — the quadratic
sections, input that neither format reads, unreadable files — raises ``MpsReadError`` carrying
the C status, and the caller falls back to samaya's own reader (the C++ binding does that,
samaya_gb300/shim/read_mps_fast.cpp).

``write_mps`` writes a ``Model`` as free MPS (samaya has no writer): rows R<i>, columns C<j>,
values by ``repr`` so that reading them back gives the same doubles.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

from . import _native
from .model import Model

SG_ERR_PARSE = -8
SG_ERR_UNSUPPORTED = -9
SG_ERR_IO = -10


class MpsReadError(RuntimeError):
    """The fast reader declined or failed; ``code`` is the SG_ERR_* status."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class _Info(ctypes.Structure):
    _fields_ = [("m", ctypes.c_int32), ("n", ctypes.c_int32), ("nnz", ctypes.c_int64),
                ("maximize", ctypes.c_int32), ("num_integers", ctypes.c_int32),
                ("obj_offset", ctypes.c_double), ("name_bytes", ctypes.c_int64),
                ("row_name_bytes", ctypes.c_int64), ("col_name_bytes", ctypes.c_int64)]


@dataclass
class MpsFile:
    """A model read from MPS: the linear model plus what samaya::Model keeps beside it."""
    model: Model
    name: str
    col_integer: np.ndarray      # uint8 per column: 1 for integer columns
    row_name_bytes: bytes
    row_name_starts: np.ndarray  # int64, m + 1
    col_name_bytes: bytes
    col_name_starts: np.ndarray  # int64, n + 1

    def row_names(self) -> list[str]:
        return _split(self.row_name_bytes, self.row_name_starts)

    def col_names(self) -> list[str]:
        return _split(self.col_name_bytes, self.col_name_starts)

    @property
    def num_integers(self) -> int:
        return int(np.count_nonzero(self.col_integer))


def _split(data: bytes, starts: np.ndarray) -> list[str]:
    s = starts.tolist()
    return [data[s[i]:s[i + 1]].decode("utf-8", "surrogateescape") for i in range(len(s) - 1)]


def _declare(lib):
    if getattr(lib, "_sg_mps_declared", False):
        return
    h = ctypes.POINTER(ctypes.c_void_p)
    P = ctypes.c_void_p
    u8 = ctypes.POINTER(ctypes.c_uint8)
    lib.sg_mps_read.restype = ctypes.c_int
    lib.sg_mps_read.argtypes = [ctypes.c_char_p, ctypes.c_int, h]
    lib.sg_mps_read_text.restype = ctypes.c_int
    lib.sg_mps_read_text.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, h]
    lib.sg_mps_get_info.restype = ctypes.c_int
    lib.sg_mps_get_info.argtypes = [P, ctypes.POINTER(_Info)]
    lib.sg_mps_get_model.restype = ctypes.c_int
    lib.sg_mps_get_model.argtypes = [P, _native.c_int64_p, _native.c_int32_p] + [
        _native.c_double_p] * 4 + [u8, _native.c_double_p, _native.c_double_p]
    lib.sg_mps_get_names.restype = ctypes.c_int
    lib.sg_mps_get_names.argtypes = [P, ctypes.c_char_p, ctypes.c_char_p, _native.c_int64_p,
                                     ctypes.c_char_p, _native.c_int64_p]
    lib.sg_mps_free.restype = None
    lib.sg_mps_free.argtypes = [P]
    lib._sg_mps_declared = True


def _lib():
    lib = _native.load()
    _declare(lib)
    return lib


def _take(lib, handle) -> MpsFile:
    """Copies a read model out of its handle (which the caller frees)."""
    info = _Info()
    lib.sg_mps_get_info(handle, ctypes.byref(info))
    m, n, nnz = info.m, info.n, info.nnz
    colptr = np.empty(n + 1, dtype=np.int64)
    rowidx = np.empty(nnz, dtype=np.int32)
    vals = np.empty(nnz, dtype=np.float64)
    obj, cl, cu = np.empty(n), np.empty(n), np.empty(n)
    integer = np.empty(n, dtype=np.uint8)
    rl, ru = np.empty(m), np.empty(m)

    def p(a, t):
        return a.ctypes.data_as(ctypes.POINTER(t))
    D = ctypes.c_double
    lib.sg_mps_get_model(handle, p(colptr, ctypes.c_int64), p(rowidx, ctypes.c_int32),
                         p(vals, D), p(obj, D), p(cl, D), p(cu, D), p(integer, ctypes.c_uint8),
                         p(rl, D), p(ru, D))
    name = ctypes.create_string_buffer(max(1, info.name_bytes))
    rn = ctypes.create_string_buffer(max(1, info.row_name_bytes))
    cn = ctypes.create_string_buffer(max(1, info.col_name_bytes))
    rs = np.empty(m + 1, dtype=np.int64)
    cs = np.empty(n + 1, dtype=np.int64)
    lib.sg_mps_get_names(handle, name, rn, p(rs, ctypes.c_int64), cn, p(cs, ctypes.c_int64))
    model = Model(m=m, n=n, colptr=colptr, rowidx=rowidx, vals=vals, obj=obj, col_lower=cl,
                  col_upper=cu, row_lower=rl, row_upper=ru, maximize=bool(info.maximize),
                  obj_offset=info.obj_offset)
    return MpsFile(model=model,
                   name=name.raw[:info.name_bytes].decode("utf-8", "surrogateescape"),
                   col_integer=integer, row_name_bytes=rn.raw[:info.row_name_bytes],
                   row_name_starts=rs, col_name_bytes=cn.raw[:info.col_name_bytes],
                   col_name_starts=cs)


def _finish(lib, rc, handle) -> MpsFile:
    if rc != 0:
        raise MpsReadError(rc, lib.sg_pdlp_last_error().decode(errors="replace"))
    try:
        return _take(lib, handle)
    finally:
        lib.sg_mps_free(handle)


def read_mps(path, threads: int = 0) -> MpsFile:
    """Reads an MPS file (threads: 0 = by the file's size; N = N ranges per section)."""
    lib = _lib()
    handle = ctypes.c_void_p()
    rc = lib.sg_mps_read(os.fsencode(path), int(threads), ctypes.byref(handle))
    return _finish(lib, rc, handle)


def read_mps_text(text, threads: int = 0) -> MpsFile:
    """Reads MPS text held in memory (str or bytes)."""
    data = text.encode() if isinstance(text, str) else bytes(text)
    lib = _lib()
    handle = ctypes.c_void_p()
    rc = lib.sg_mps_read_text(data, len(data), int(threads), ctypes.byref(handle))
    return _finish(lib, rc, handle)


def mps_lines(model: Model, name: str = "model", col_integer=None, two_per_line: bool = True):
    """The lines of a free-MPS file of ``model``: rows E / L / G (two-sided rows as G rows with
    a range, which reads back as lower + (upper - lower); a free row as an L row with RHS inf),
    bounds LO / UP / MI / FR / FX, integer markers from ``col_integer``, OBJSENSE MAX for a
    maximisation, the offset as the objective's RHS."""
    m, n = model.m, model.n
    rl, ru = model.row_lower, model.row_upper
    rname = [f"R{i}" for i in range(m)]
    lines = [f"NAME {name}"]
    if model.maximize:
        lines += ["OBJSENSE", "    MAX"]
    lines += ["ROWS", " N obj"]
    rhs, ranges = [], []
    for i in range(m):
        lo, up = float(rl[i]), float(ru[i])
        if lo == up:
            lines.append(f" E {rname[i]}")
            rhs.append((rname[i], lo))
        elif np.isinf(lo):
            lines.append(f" L {rname[i]}")
            rhs.append((rname[i], up))
        elif np.isinf(up):
            lines.append(f" G {rname[i]}")
            rhs.append((rname[i], lo))
        else:
            lines.append(f" G {rname[i]}")
            rhs.append((rname[i], lo))
            ranges.append((rname[i], up - lo))
    lines.append("COLUMNS")
    colptr, rowidx = model.colptr.tolist(), model.rowidx.tolist()
    vals = list(map(repr, model.vals.tolist()))
    obj = model.obj.tolist()
    integer = None if col_integer is None else np.asarray(col_integer).tolist()
    in_int = False
    for j in range(n):
        if integer is not None and bool(integer[j]) != in_int:
            in_int = bool(integer[j])
            lines.append(f"    M{j} 'MARKER' '{'INTORG' if in_int else 'INTEND'}'")
        c = f" C{j}"
        ents = [f"{rname[rowidx[p]]} {vals[p]}" for p in range(colptr[j], colptr[j + 1])]
        if obj[j] != 0.0:
            ents.insert(0, f"obj {obj[j]!r}")
        if not ents:
            ents = ["obj 0.0"]
        step = 2 if two_per_line else 1
        for k in range(0, len(ents), step):
            lines.append(c + " " + " ".join(ents[k:k + step]))
    if in_int:
        lines.append("    MEND 'MARKER' 'INTEND'")
    lines.append("RHS")
    if model.obj_offset != 0.0:
        lines.append(f" rhs obj {-model.obj_offset!r}")
    lines += [f" rhs {r} {v!r}" for r, v in rhs if v != 0.0]
    if ranges:
        lines.append("RANGES")
        lines += [f" rng {r} {v!r}" for r, v in ranges]
    lines.append("BOUNDS")
    cl, cu = model.col_lower.tolist(), model.col_upper.tolist()
    for j in range(n):
        lo, up = cl[j], cu[j]
        if lo == up:
            lines.append(f" FX bnd C{j} {lo!r}")
            continue
        if lo == -np.inf and up == np.inf:
            lines.append(f" FR bnd C{j}")
            continue
        if lo == -np.inf:
            lines.append(f" MI bnd C{j}")
        elif lo != 0.0 or up < 0.0:  # UP < 0 alone would make the lower bound -inf
            lines.append(f" LO bnd C{j} {lo!r}")
        if up != np.inf:
            lines.append(f" UP bnd C{j} {up!r}")
    lines.append("ENDATA")
    return lines


def write_mps(model: Model, path, name: str = "model", col_integer=None) -> None:
    """Writes ``model`` as a free-MPS file (see ``mps_lines``)."""
    with open(path, "w") as f:
        f.write("\n".join(mps_lines(model, name, col_integer)))
        f.write("\n")
