"""The fast MPS reader (include/sg_mps.h) against samaya's own reader (samaya::read_mps,
reference src/io/mps_reader.cpp): bit for bit on every case of tests/golden/mps_cases.py, through
the committed fixture tests/golden/mps_golden.npz (made by make_mps_golden.py from samaya's
reader) and, where the samaya checkout is present, against samaya's reader run here; the same
refusals; several thread counts, so that sections are cut into ranges inside columns, integer
blocks and repeated columns; and the full-size transportation LP (1000 x 2000, a 93 MB file).
Host code only: no GPU."""
from __future__ import annotations

import os
import re
import sys

import numpy as np
import pytest

from samaya_gb300 import generators as g
from samaya_gb300 import mps

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
from mps_cases import accepted_cases, rejected_cases  # noqa: E402

GOLDEN = np.load(os.path.join(HERE, "golden", "mps_golden.npz"))
THREADS = (0, 1, 3, 8, 17)
ARRAYS = ("colptr", "rowidx", "vals", "obj", "col_lower", "col_upper", "row_lower", "row_upper")


def _bits(a):
    a = np.ascontiguousarray(a)
    return a.view(np.uint8) if a.size else a


def _fast_dict(f: mps.MpsFile) -> dict:
    md = f.model
    d = {k: getattr(md, k) for k in ARRAYS}
    d.update(col_integer=f.col_integer, row_starts=f.row_name_starts,
             col_starts=f.col_name_starts, m=md.m, n=md.n, maximize=md.maximize,
             obj_offset=md.obj_offset, name=f.name.encode("utf-8", "surrogateescape"),
             row_names=f.row_name_bytes, col_names=f.col_name_bytes)
    return d


def _assert_same(got: dict, want: dict, what: str):
    assert (got["m"], got["n"], bool(got["maximize"])) == (want["m"], want["n"],
                                                           bool(want["maximize"])), what
    assert _bits(np.float64(got["obj_offset"])).tobytes() == \
        _bits(np.float64(want["obj_offset"])).tobytes(), what
    for k in ARRAYS + ("col_integer", "row_starts", "col_starts"):
        a, b = np.asarray(got[k]), np.asarray(want[k])
        assert a.shape == b.shape, (what, k, a.shape, b.shape)
        assert np.array_equal(_bits(a.astype(b.dtype)), _bits(b)), (what, k)
    for k in ("name", "row_names", "col_names"):
        assert bytes(got[k]) == bytes(want[k]), (what, k)


def _golden(name: str) -> dict:
    d = {k: GOLDEN[f"{name}__{k}"] for k in ARRAYS + ("col_integer", "row_starts",
                                                       "col_starts")}
    m, n, mx = (int(v) for v in GOLDEN[f"{name}__meta"])
    d.update(m=m, n=n, maximize=bool(mx), obj_offset=float(GOLDEN[f"{name}__offset"][0]))
    for k in ("name", "row_names", "col_names"):
        d[k] = GOLDEN[f"{name}__{k}"].tobytes()
    return d


def _ref():
    from oracle import ref
    if not ref.available():
        pytest.skip("the samaya checkout is not present")
    ref.build()
    return ref


@pytest.mark.parametrize("threads", THREADS)
def test_accepted_cases_match_the_golden_fixture(threads):
    for name, text in accepted_cases():
        got = _fast_dict(mps.read_mps_text(text, threads=threads))
        _assert_same(got, _golden(name), f"{name} threads={threads}")


def test_accepted_cases_match_samayas_reader():
    ref = _ref()
    for name, text in accepted_cases():
        want = ref.mps_read_text(text)
        for threads in (0, 2, 5):
            _assert_same(_fast_dict(mps.read_mps_text(text, threads=threads)), want,
                         f"{name} threads={threads}")


def _line(message: str) -> int:
    m = re.match(r"line (\d+): ", message)
    return int(m.group(1)) if m else 0


@pytest.mark.parametrize("threads", (0, 1, 4))
def test_rejected_cases(threads):
    """Every input that free MPS rejects is refused with SG_ERR_PARSE at the line samaya's reader
    names (0 for the whole-model checks); the quadratic sections with SG_ERR_UNSUPPORTED. Where
    samaya's reader goes on to read the text (fixed MPS, quadratic sections), the caller's
    fallback does the same."""
    codes = {"parse": mps.SG_ERR_PARSE, "unsupported": mps.SG_ERR_UNSUPPORTED}
    for name, text, status, samaya in rejected_cases():
        with pytest.raises(mps.MpsReadError) as e:
            mps.read_mps_text(text, threads=threads)
        assert e.value.code == codes[status], (name, str(e.value))
        raises, line = (int(v) for v in GOLDEN[f"rejected__{name}"])
        assert raises == (samaya == "raises"), name
        if raises:
            assert _line(str(e.value)) == line, (name, str(e.value), line)


def test_rejected_cases_against_samayas_reader():
    ref = _ref()
    for name, text, _, samaya in rejected_cases():
        try:
            ref.mps_read_text(text)
            got = "reads"
        except ref.RefMpsError:
            got = "raises"
        assert got == samaya, name


def test_round_trip_of_generated_models():
    """write_mps then read_mps gives back the model's arrays exactly (models without two-sided
    rows, whose range reads back as lower + (upper - lower))."""
    for model in (g.random_sparse_lp(300, 800, seed=3), g.transportation_lp(30, 70, seed=1),
                  g.power_law_lp(m=2000, n=4000, seed=5), g.facility_location_lp(10, 40, seed=2)):
        f = mps.read_mps_text("\n".join(mps.mps_lines(model)) + "\n", threads=3)
        for k in ARRAYS:
            assert np.array_equal(_bits(getattr(f.model, k)), _bits(getattr(model, k))), k
        assert f.model.maximize == model.maximize
        assert f.row_names() == [f"R{i}" for i in range(model.m)]
        assert f.col_names()[:3] == ["C0", "C1", "C2"]


def test_file_and_text_agree(tmp_path):
    model = g.random_sparse_lp(200, 500, seed=9)
    path = tmp_path / "lp.mps"
    mps.write_mps(model, path)
    a = _fast_dict(mps.read_mps(path))
    b = _fast_dict(mps.read_mps_text(path.read_bytes(), threads=5))
    _assert_same(a, b, "file vs text")
    with pytest.raises(mps.MpsReadError) as e:
        mps.read_mps(tmp_path / "missing.mps")
    assert e.value.code == mps.SG_ERR_IO


def test_many_ranges_on_a_small_file():
    """More ranges than lines in a section: empty ranges, cuts moved past whole columns."""
    text = dict(accepted_cases())["markers"]
    want = _golden("markers")
    for threads in (32, 64):
        _assert_same(_fast_dict(mps.read_mps_text(text, threads=threads)), want, str(threads))


def test_full_size_transportation_lp(tmp_path):
    """The transportation LP of the benchmark (3,000 rows, 2,000,000 columns, 4,000,000
    entries; a 93 MB file): the same model as samaya's reader, and the generator's arrays."""
    model = g.transportation_lp(1000, 2000, seed=0)
    path = tmp_path / "transport.mps"
    mps.write_mps(model, path)
    f = mps.read_mps(path)
    for k in ARRAYS:
        assert np.array_equal(_bits(getattr(f.model, k)), _bits(getattr(model, k))), k
    try:
        ref = _ref()
    except pytest.skip.Exception:
        return
    _assert_same(_fast_dict(f), ref.mps_read_file(path), "transport 1000 x 2000")


def test_samayas_own_test_inputs():
    """The MPS inputs of samaya's own reader tests: the complete texts in
    tests/test_mps_reader.cpp and the files of tests/instances (a MIPLIB instance with integer
    markers, a crude-blending LP, pooling problems with QCMATRIX rows), read from the samaya
    checkout at test time. The linear ones read to samaya's Model bit for bit; the quadratic
    ones are declined for samaya's reader to take."""
    import glob
    from oracle import ref
    root = ref.REFERENCE_ROOT
    src = os.path.join(root, "tests", "test_mps_reader.cpp")
    if not os.path.exists(src):
        pytest.skip("the samaya checkout is not present")
    ref.build()
    with open(src) as f:
        texts = [t for t in re.findall(r'R"\((.*?)\)"', f.read(), re.S)
                 if t.lstrip().startswith("NAME")]
    inputs = [(f"test_mps_reader.cpp #{i}", t.encode()) for i, t in enumerate(texts)]
    for p in sorted(glob.glob(os.path.join(root, "tests", "instances", "*.mps"))):
        with open(p, "rb") as f:
            inputs.append((os.path.basename(p), f.read()))
    linear = quadratic = 0
    for name, text in inputs:
        want = ref.mps_read_text(text)
        if want["q_nnz"] or want["quadratic_rows"]:
            with pytest.raises(mps.MpsReadError) as e:
                mps.read_mps_text(text, threads=3)
            assert e.value.code == mps.SG_ERR_UNSUPPORTED, name
            quadratic += 1
            continue
        for threads in (0, 3):
            _assert_same(_fast_dict(mps.read_mps_text(text, threads=threads)), want, name)
        linear += 1
    assert linear >= 7 and quadratic >= 3, (linear, quadratic)
