"""The engine library's host code under AddressSanitizer and UBSan (CPU test): samaya_gb300.build's
sanitizer variant (built into a temporary directory) runs the host-only test files — the tile
partition, every C entry that needs no GPU (input checks, sg_scale_model, sg_csc_to_csr, the
batch checks, sg_build_tiles), the MPS reader with its random and mutated texts, and the oracle
pins that go through sg_scale_model — with the sanitizer runtimes preloaded. No report, every
test passing."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
FILES = ("test_tiles.py", "test_cabi.py", "test_mps.py", "test_mps_fuzz.py",
         "test_oracle_pin.py")


def _runtime(name):
    p = subprocess.run(["gcc", f"-print-file-name={name}"], capture_output=True, text=True)
    path = p.stdout.strip()
    return path if os.path.isabs(path) and os.path.exists(path) else None


def test_host_code_is_clean_under_sanitizers(tmp_path):
    if shutil.which("gcc") is None or shutil.which("nvcc") is None and not os.path.exists(
            "/usr/local/cuda/bin/nvcc"):
        pytest.skip("no gcc or nvcc")
    asan, ubsan, cxx = (_runtime(n) for n in ("libasan.so", "libubsan.so", "libstdc++.so"))
    if asan is None or ubsan is None or cxx is None:
        pytest.skip("no sanitizer runtime")
    from samaya_gb300 import build
    lib = build.build_sanitized(str(tmp_path / "asan"))
    # libstdc++ is preloaded too: ASan's exception interceptor needs it before the library's
    # first throw in a Python process.
    env = dict(os.environ, SAMAYA_GB300_LIB=lib, LD_PRELOAD=f"{asan} {ubsan} {cxx}",
               ASAN_OPTIONS="detect_leaks=0:halt_on_error=1",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1", CUDA_VISIBLE_DEVICES="")
    run = subprocess.run([sys.executable, "-m", "pytest", "-x", "-q", "-s", "-p",
                          "no:cacheprovider", "-m", "not gpu",
                          *[os.path.join(HERE, f) for f in FILES]],
                         cwd=ROOT, env=env, capture_output=True, text=True, timeout=1800)
    out = run.stdout + run.stderr
    assert "ERROR: AddressSanitizer" not in out and "runtime error" not in out, out[-4000:]
    assert run.returncode == 0, out[-4000:]
