"""The model setup on the device (sg_scale_model_device, sg_pdlp_create_model): samaya's
compute_scaling + make_problem and the engine's row-major copy computed on the GPU give the bits
the host code gives (sg_scale_model, pinned to the reference's own LpProblem fixtures, and the
host transpose), so a solve from the device-built problem repeats the host-built solve bit for
bit."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GROUPS, load_group

pytestmark = pytest.mark.gpu


def _models():
    from samaya_gb300 import generators as g
    out = []
    for group in GROUPS:
        out += [c.model for c in load_group(group)]
    out += [g.random_sparse_lp(2000, 5000, seed=0), g.transportation_lp(100, 200, seed=3),
            g.facility_location_lp(20, 60, seed=3), g.power_law_lp(m=20000, n=40000, seed=2)]
    return out


def test_device_scaling_matches_the_host_bit_for_bit(engine):
    """Every output of sg_scale_model_device equals sg_scale_model's on the models of every
    fixture group (the reference's own LP families; the host output equals the reference's
    LpProblem there) and on random sparse, transportation, facility-location and power-law
    models."""
    from samaya_gb300.problem import make_problem
    checked = 0
    for model in _models():
        host, hs = make_problem(model)
        dev, ds = make_problem(model, device=True)
        for k in ("colptr", "rowidx", "vals", "cost", "lower", "upper"):
            assert np.array_equal(getattr(host, k), getattr(dev, k)), (model.m, model.n, k)
        assert np.array_equal(hs.col, ds.col) and np.array_equal(hs.row, ds.row)
        checked += 1
    assert checked > 100


@pytest.mark.parametrize("name", ["random", "transport", "powerlaw"])
def test_engine_from_a_device_built_problem_repeats_the_host_solve(engine, name):
    """sg_pdlp_create_model (scaling, computational form and the CSC -> CSR transpose on the
    device) against sg_pdlp_create on the host-built LpProblem: the same scale factors and a
    bit-identical solve (status, iterations, x, y)."""
    from samaya_gb300 import generators as g
    from samaya_gb300.problem import make_problem
    model = {"random": lambda: g.random_sparse_lp(500, 1200, seed=4),
             "transport": lambda: g.transportation_lp(100, 200, seed=3),
             "powerlaw": lambda: g.power_law_lp(m=20000, n=40000, seed=2)}[name]()
    opts = engine.PdlpOptions(tol=1e-6, precision=engine.FP32_THEN_FP64,
                              algorithm=engine.HALPERN, inner_tol=1e-5, autotune=False)
    lp, sc = make_problem(model)
    with engine.PdlpSolver(lp, opts) as s:
        a = s.solve()
    with engine.PdlpSolver.from_model(model, opts) as s:
        b = s.solve()
        assert np.array_equal(s.scaling.col, sc.col) and np.array_equal(s.scaling.row, sc.row)
    assert a.status == b.status and a.iterations == b.iterations
    assert np.array_equal(a.x, b.x) and np.array_equal(a.y, b.y)


def test_device_setup_rejects_bad_input(engine):
    """A row index out of range or a value that is not finite is found on the device and
    refused before anything uses it (SG_ERR_INVALID_ARGUMENT)."""
    from samaya_gb300 import _native
    from samaya_gb300.generators import random_sparse_lp
    from samaya_gb300.model import Model
    from samaya_gb300.problem import make_problem
    base = random_sparse_lp(50, 120, seed=1)
    for field, value in (("rowidx", 50), ("vals", np.inf)):
        arr = getattr(base, field).copy()
        arr[7] = value
        bad = Model(**{**base.__dict__, field: arr})
        with pytest.raises(_native.EngineError) as info:
            make_problem(bad, device=True)
        assert info.value.code == -1
