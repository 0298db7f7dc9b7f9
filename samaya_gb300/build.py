"""Build recipe of the engine's shared library (in-tree, no cmake).

Compiles every translation unit under ``samaya_gb300/csrc`` for sm_103a with nvcc, in parallel,
and links ``samaya_gb300/_lib/libsamaya_gb300.so`` (CUDA runtime linked statically, so the
library needs only the driver).
"""
from __future__ import annotations

import concurrent.futures
import glob
import hashlib
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB_PATH = os.path.join(OUT_DIR, "libsamaya_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _sources():
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers():
    return sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
                  glob.glob(os.path.join(HERE, "..", "include", "*.h")))


def _digest(paths) -> str:
    h = hashlib.sha256()
    for p in paths:
        h.update(p.encode())
        with open(p, "rb") as f:
            h.update(f.read())
    return h.hexdigest()


def _compile(src: str, flags, obj_dir: str = OBJ_DIR, opt=("-O3", "-Xcompiler", "-O2")) -> str:
    obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
    cmd = [nvcc_path(), *ARCH, opt[0], "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
           *opt[1:], "-I", os.path.join(HERE, "..", "include"), *flags, "-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc_path(), "-x", "cu", *cmd[1:]]
    subprocess.run(cmd, check=True)
    return obj


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Builds the library if a source or header changed; returns its path."""
    srcs = _sources()
    stamp_path = os.path.join(OUT_DIR, "stamp")
    digest = _digest(srcs + _headers()) + "|" + " ".join(extra_flags)
    if not force and os.path.exists(LIB_PATH) and os.path.exists(stamp_path):
        with open(stamp_path) as f:
            if f.read() == digest:
                return LIB_PATH
    os.makedirs(OBJ_DIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, list(extra_flags)), srcs))
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.run([nvcc_path(), *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static",
                    "-lpthread"], check=True)
    os.replace(tmp, LIB_PATH)
    with open(stamp_path, "w") as f:
        f.write(digest)
    if verbose:
        print("built", LIB_PATH)
    return LIB_PATH


def build_sanitized(out_dir: str) -> str:
    """The same library with AddressSanitizer and UBSan in its host code (-O1, -g), linked into
    out_dir, never in-tree: for tests that run the host-only entry points under the sanitizers
    (load it with SAMAYA_GB300_LIB and the sanitizer runtimes preloaded). Returns its path."""
    obj_dir = os.path.join(out_dir, "obj")
    os.makedirs(obj_dir, exist_ok=True)
    san = ["-g", "-Xcompiler",
           "-fsanitize=address,-fsanitize=undefined,-fno-sanitize-recover=all,"
           "-fno-omit-frame-pointer"]
    srcs = _sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, san, obj_dir, ("-O1",)), srcs))
    path = os.path.join(out_dir, "libsamaya_gb300.so")
    subprocess.run([nvcc_path(), *ARCH, "-shared", "-o", path, *objs, "-cudart", "static",
                    "-lpthread", "-Xcompiler", "-fsanitize=address,-fsanitize=undefined"],
                   check=True)
    return path


if __name__ == "__main__":
    build(force=True, verbose=True)
