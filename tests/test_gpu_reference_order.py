"""The FP64 path in the reference's order of operations (order="reference",
PLSQR_ORDER_REFERENCE): every product, sum and norm evaluated as the
reference's CPU code does, so that a solve returns the reference's bits.

Checked bit for bit against the reference program's own golden runs (x,
alpha_k, beta_k, result.txt) and against the oracle, which reproduces the
reference bit for bit (per-iteration rnorm, arnorm, anorm, acond, xnorm,
test1, test2; damped solves; se; the operator alone)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

SCALARS = ("alpha", "beta", "rnorm", "arnorm", "test1", "test2", "anorm", "acond", "xnorm")


@pytest.mark.parametrize("case", ["tiny", "grid32"])
def test_reference_order_reproduces_reference_bits(case, pkg, orc, problems, tmp_path):
    g = golden(case)
    prob = problems(case)
    it = g["meta"]["iterations"]
    with pkg.Context(prob, order="reference") as ctx:
        out = ctx.lsqr(lsqr_iteration=it, result_txt=str(tmp_path / "result.txt"))
    assert np.array_equal(out["x"], g["x"])
    assert np.array_equal(out["hist"]["alpha"], g["alpha"])
    assert np.array_equal(out["hist"]["beta"], g["beta"])
    assert (tmp_path / "result.txt").read_text() == g["result_txt"]
    ref = orc.OracleProblem(prob).lsqr(it)
    for k in SCALARS:
        assert np.array_equal(out["hist"][k][1:], ref["hist"][k][1:]), k
    for k in ("rnorm", "xnorm", "anorm", "acond", "arnorm_out", "istop", "itn"):
        assert out["result"][k] == ref["result"][k], k


@pytest.mark.parametrize("damp,want_se", [(0.3, False), (0.0, True), (0.7, True)])
def test_reference_order_damped_and_se_bitwise(damp, want_se, pkg, orc, problems):
    prob = problems("grid32")
    it = 60
    with pkg.Context(prob, order="reference") as ctx:
        out = ctx.lsqr(lsqr_iteration=it, damp=damp, want_se=want_se)
    ref = orc.OracleProblem(prob).lsqr(it, damp=damp, want_se=want_se)
    assert np.array_equal(out["x"], ref["x"])
    for k in SCALARS:
        assert np.array_equal(out["hist"][k][1:], ref["hist"][k][1:]), k
    if want_se:
        assert np.array_equal(out["se"], ref["se"])
    assert out["result"]["istop"] == ref["result"]["istop"]


@pytest.mark.parametrize("case", ["tiny", "grid32"])
def test_reference_order_aprod_bitwise(case, pkg, orc, problems):
    prob = problems(case)
    rng = np.random.default_rng(11)
    with pkg.Context(prob, order="reference") as ctx:
        for mode in (1, 2):
            yk, yd = rng.standard_normal(prob.m_k), rng.standard_normal(prob.m_d)
            x = rng.standard_normal(prob.n)
            o = orc.OracleProblem(prob)
            o.y_k[:], o.y_d[:], o.x[:] = yk, yd, x
            o.aprod(mode)
            ctx.aprod_host(mode, yk, yd, x)
            assert np.array_equal(yk, o.y_k) and np.array_equal(yd, o.y_d)
            assert np.array_equal(x, o.x)


def test_reference_order_zero_rhs_and_short_runs(pkg, orc, problems):
    prob = problems("tiny")
    with pkg.Context(prob, order="reference") as ctx:
        z = ctx.lsqr(np.zeros(prob.m_k), lsqr_iteration=5)
        assert np.array_equal(z["x"], np.zeros(prob.n))
        for it in (0, 1, 2):
            out = ctx.lsqr(lsqr_iteration=it)
            ref = orc.OracleProblem(prob).lsqr(it)
            assert np.array_equal(out["x"], ref["x"]), it
            assert np.array_equal(out["hist"]["alpha"], ref["hist"]["alpha"]), it


def test_reference_order_graph_and_stream_agree(pkg, problems):
    prob = problems("grid32")
    outs = []
    for graph in (True, False):
        with pkg.Context(prob, order="reference", use_graph=graph) as ctx:
            outs.append(ctx.lsqr(lsqr_iteration=20))
    assert np.array_equal(outs[0]["x"], outs[1]["x"])
    assert np.array_equal(outs[0]["hist"]["beta"], outs[1]["hist"]["beta"])


def test_reference_order_refuses_mixed_precision(pkg, problems):
    with pytest.raises(RuntimeError):
        pkg.Context(problems("tiny"), order="reference", precision="mixed")
