"""ctypes binding of the engine's C ABI (include/sg_pdlp.h).

The library is built in-tree by ``samaya_gb300.build``; loading fails loudly when it is missing
or when no usable GPU is present — there is no CPU fallback on this path.
"""
from __future__ import annotations

import ctypes
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
# SAMAYA_GB300_LIB names another build of the library to load (a sanitizer build in tests).
LIB_PATH = os.environ.get("SAMAYA_GB300_LIB") or os.path.join(_HERE, "_lib", "libsamaya_gb300.so")
HEADER = os.path.join(_HERE, "..", "include", "sg_pdlp.h")

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int64_p = ctypes.POINTER(ctypes.c_int64)
c_int32_p = ctypes.POINTER(ctypes.c_int32)


class Opts(ctypes.Structure):
    _fields_ = [("tol", ctypes.c_double), ("max_iterations", ctypes.c_longlong),
                ("time_limit", ctypes.c_double), ("precision", ctypes.c_int),
                ("refine_max_rounds", ctypes.c_int), ("inner_tol", ctypes.c_double),
                ("verbose", ctypes.c_int), ("algorithm", ctypes.c_int),
                ("autotune", ctypes.c_int),
                ("tile_split", ctypes.c_int), ("artificial_restart", ctypes.c_double),
                ("keep_inert_rows", ctypes.c_int), ("row_groups", ctypes.c_int),
                ("segment_staging", ctypes.c_int), ("tile_nnz", ctypes.c_int)]


class Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_longlong),
                ("primal_residual", ctypes.c_double), ("dual_residual", ctypes.c_double),
                ("gap", ctypes.c_double), ("primal_objective", ctypes.c_double),
                ("dual_objective", ctypes.c_double), ("restarts", ctypes.c_longlong),
                ("evaluations", ctypes.c_longlong), ("refinement_rounds", ctypes.c_int),
                ("has_dual_ray", ctypes.c_int), ("has_primal_ray", ctypes.c_int),
                ("setup_seconds", ctypes.c_double), ("solve_seconds", ctypes.c_double),
                ("step_size", ctypes.c_double), ("primal_weight", ctypes.c_double),
                ("kernel_launches", ctypes.c_longlong), ("device_ms", ctypes.c_double)]


_lib = None


def declared_symbols():
    """Function names declared in include/*.h."""
    names = []
    inc = os.path.join(_HERE, "..", "include")
    for fn in sorted(os.listdir(inc)):
        if not fn.endswith(".h"):
            continue
        with open(os.path.join(inc, fn)) as f:
            text = f.read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(sg_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def load(build_if_missing: bool = False):
    """Loads the engine library (building it first if asked)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from . import build
            build.build()
        else:
            raise RuntimeError(
                f"samaya_gb300: the CUDA library {LIB_PATH} is not built; run "
                "`python -c 'import __graft_entry__ as g; g.build()'` first")
    lib = ctypes.CDLL(LIB_PATH)
    _declare(lib)
    _lib = lib
    return lib


def _declare(lib):
    I, D, LL, P = ctypes.c_int, ctypes.c_double, ctypes.c_longlong, ctypes.c_void_p
    h = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "sg_pdlp_default_opts": (None, [ctypes.POINTER(Opts)]),
        "sg_pdlp_available": (I, [ctypes.POINTER(I), ctypes.POINTER(I), ctypes.c_char_p,
                                  ctypes.c_size_t]),
        "sg_pdlp_create": (I, [h, I, I, c_int64_p, c_int32_p, c_double_p, c_double_p, c_double_p,
                               c_double_p, ctypes.POINTER(Opts)]),
        "sg_pdlp_solve": (I, [P, ctypes.POINTER(Result), c_double_p, c_double_p, c_double_p,
                              c_double_p]),
        "sg_pdlp_destroy": (None, [P]),
        "sg_pdlp_error_string": (ctypes.c_char_p, [I]),
        "sg_pdlp_last_error": (ctypes.c_char_p, []),
        "sg_pdlp_solve_problem": (I, [I, I, c_int64_p, c_int32_p, c_double_p, c_double_p,
                                      c_double_p, c_double_p, ctypes.POINTER(Opts),
                                      ctypes.POINTER(Result), c_double_p, c_double_p, c_double_p,
                                      c_double_p]),
        "sg_pdhg_create": (I, [h, I, I, c_int64_p, c_int32_p, c_double_p, c_double_p, c_double_p,
                               c_double_p]),
        "sg_pdhg_set_original": (I, [P, c_double_p, c_double_p, c_double_p, c_double_p,
                                     c_double_p]),
        "sg_pdhg_step": (I, [P, D, D, D, LL]),
        "sg_pdhg_advance": (I, [P]),
        "sg_pdhg_evaluate": (I, [P, I, c_double_p]),
        "sg_pdhg_restart_distance": (I, [P, I, c_double_p, c_double_p]),
        "sg_pdhg_restart_to": (I, [P, I]),
        "sg_pdhg_download": (I, [P, c_double_p, c_double_p, c_double_p, c_double_p, c_double_p,
                                 c_double_p]),
        "sg_pdlp_equilibration": (I, [P, c_double_p, c_double_p, c_double_p, c_double_p]),
        "sg_pdhg_set_state": (I, [P, I, c_double_p, c_double_p, c_double_p, c_double_p]),
        "sg_pdhg_halpern_step": (I, [P, D, D, LL]),
        "sg_spmv": (I, [P, I, c_double_p, c_double_p]),
        "sg_pdlp_time_kernels": (I, [P, I, c_double_p, c_double_p, c_double_p]),
        "sg_pdlp_tile_shape": (I, [P, I] + [ctypes.POINTER(ctypes.c_int)] * 5),
        "sg_pdlp_step_rows": (I, [P] + [ctypes.POINTER(ctypes.c_int)] * 4),
        "sg_build_tiles": (I, [I, c_int32_p, I, I, I, I, c_int32_p, I,
                               ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
        "sg_build_group_tiles": (I, [I, c_int32_p, ctypes.POINTER(ctypes.c_uint8), I, I, I, I,
                                     c_int32_p, I, ctypes.POINTER(ctypes.c_int),
                                     ctypes.POINTER(ctypes.c_int)]),
        "sg_csc_to_csr": (I, [I, I, c_int64_p, c_int32_p, c_double_p, c_int32_p, c_int32_p,
                              c_double_p]),
        "sg_scale_model": (I, [I, I, c_int64_p, c_int32_p, c_double_p, c_double_p, c_double_p,
                               c_double_p, c_double_p, c_double_p, I, c_int64_p, c_int32_p,
                               c_double_p, c_double_p, c_double_p, c_double_p, c_double_p,
                               c_double_p, c_int64_p]),
        "sg_unscale_solution": (I, [I, I, c_double_p, c_double_p, I, c_double_p, c_double_p,
                                    c_double_p, c_double_p, c_double_p]),
        "sg_scale_model_device": (I, [I, I, c_int64_p, c_int32_p, c_double_p, c_double_p,
                                      c_double_p, c_double_p, c_double_p, c_double_p, I,
                                      c_int64_p, c_int32_p, c_double_p, c_double_p, c_double_p,
                                      c_double_p, c_double_p, c_double_p, c_int64_p]),
        "sg_pdlp_create_model": (I, [h, I, I, c_int64_p, c_int32_p, c_double_p, c_double_p,
                                     c_double_p, c_double_p, c_double_p, c_double_p, I,
                                     ctypes.POINTER(Opts), c_double_p, c_double_p]),
    }
    for name, (res, args) in sig.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args


class EngineError(RuntimeError):
    def __init__(self, code, where):
        lib = load()
        msg = lib.sg_pdlp_last_error().decode() or lib.sg_pdlp_error_string(code).decode()
        super().__init__(f"{where}: {msg} (code {code})")
        self.code = code


def check(code, where):
    if code != 0:
        raise EngineError(code, where)
