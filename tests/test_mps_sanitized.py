"""The fast MPS reader's host code under AddressSanitizer and UBSan (CPU test): sg_mps.cpp built
with -fsanitize=address,undefined together with tests/c/mps_sanitize_driver.cpp and run on every
case of tests/golden/mps_cases.py, the seeded random, fixed-format and byte-mutated texts of
test_mps_fuzz.py, and a generated power-law LP of 1.2M entries, each at 1, 3 and 7 threads. No
sanitizer report, and the same status, sizes and checksum at every thread count."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from collections import defaultdict

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(HERE, "golden"))
sys.path.insert(0, HERE)


def test_reader_is_clean_under_sanitizers(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    from mps_cases import accepted_cases, rejected_cases
    from test_mps_fuzz import _fixed_text, _mutated, _text
    from samaya_gb300 import generators as g
    from samaya_gb300.mps import write_mps
    exe = tmp_path / "mps_sanitize"
    csrc = os.path.join(ROOT, "samaya_gb300", "csrc")
    build = subprocess.run(
        ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
         "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-pthread", "-I", csrc,
         os.path.join(csrc, "sg_mps.cpp"), os.path.join(HERE, "c", "mps_sanitize_driver.cpp"),
         "-o", str(exe)], capture_output=True, text=True)
    if build.returncode != 0 and "sanitize" in build.stderr:
        pytest.skip("the compiler has no sanitizer runtime")
    assert build.returncode == 0, build.stderr
    texts = [t.encode() for _, t in accepted_cases()]
    texts += [case[1].encode() for case in rejected_cases()]
    texts += [_text(s).encode() for s in range(100)] + [_mutated(s) for s in range(300)]
    texts += [_fixed_text(s).encode() for s in range(100)]
    paths = []
    for k, t in enumerate(texts):
        p = tmp_path / f"t{k}.mps"
        p.write_bytes(t)
        paths.append(str(p))
    big = tmp_path / "powerlaw.mps"
    write_mps(g.power_law_lp(m=100_000, n=200_000, seed=2), big)
    paths.append(str(big))
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:halt_on_error=1",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    run = subprocess.run([str(exe)], input="\n".join(paths) + "\n", capture_output=True,
                         text=True, env=env, timeout=1200)
    assert run.returncode == 0 and "runtime error" not in run.stderr, run.stderr[-3000:]
    seen = defaultdict(set)
    for line in run.stdout.splitlines():
        path, _, status, n, nnz, checksum, err_line = line.split()
        seen[path].add((status, n, nnz, checksum, err_line))
    assert len(seen) == len(paths)
    assert all(len(v) == 1 for v in seen.values()), [p for p, v in seen.items() if len(v) != 1]
