"""Parity on the reference's own data: the first 25 rays of its data/ sample
(Southern California, 99 x 153 x 10 cells, 2 parameter fields, 302,940
columns, the README's damping matrix: 1,910,672 rows) solved for 100
iterations as data/LSQR_run/LSQR3.pbs runs it.  The golden run is the
reference program's on kernel files made by the reference's own tools
(tests/golden/socal25, see make_golden.py)."""
from __future__ import annotations

import hashlib
import json

import numpy as np
import pytest

from conftest import GOLDEN, rel

pytestmark = pytest.mark.gpu

SOCAL = GOLDEN / "socal25"
HIST_KEYS = ("rnorm", "arnorm", "anorm", "xnorm", "test1", "test2")


@pytest.fixture(scope="module")
def socal(pkg):
    z = np.load(SOCAL / "rays.npz")
    prob = pkg.raykernels.socal_from_rays(pkg.raykernels.socal_from_compact(z), z["b_k"])
    meta = json.loads((SOCAL / "meta.json").read_text())
    ab = np.loadtxt(SOCAL / "alpha_beta.txt")
    h = np.loadtxt(SOCAL / "hist.txt")
    gold = dict(alpha=ab[:, 1], beta=ab[:, 2], **{k: h[:, 1 + i] for i, k in enumerate(HIST_KEYS)})
    return prob, meta, gold


def test_socal_reference_order_bitwise(pkg, socal, tmp_path):
    prob, meta, gold = socal
    it = meta["iterations"]
    with pkg.Context(prob, order="reference") as ctx:
        out = ctx.lsqr(lsqr_iteration=it, result_txt=str(tmp_path / "result.txt"))
    assert hashlib.sha256(out["x"].tobytes()).hexdigest() == meta["x_sha256"]
    for k in ("alpha", "beta"):
        assert np.array_equal(out["hist"][k], gold[k]), k
    for k in HIST_KEYS:
        assert np.array_equal(out["hist"][k][1:], gold[k][1:]), k
    assert (tmp_path / "result.txt").read_text() == (SOCAL / "result.txt").read_text()


def test_socal_fast_order_within_tolerance(pkg, socal):
    prob, meta, gold = socal
    it = meta["iterations"]
    with pkg.Context(prob, order="reference") as ctx:
        ref = ctx.lsqr(lsqr_iteration=it)
    assert hashlib.sha256(ref["x"].tobytes()).hexdigest() == meta["x_sha256"]
    with pkg.Context(prob) as ctx:
        out = ctx.lsqr(lsqr_iteration=it)
    assert rel(out["x"], ref["x"]) <= 1e-10
    for k in ("rnorm", "xnorm"):
        assert abs(out["hist"][k][-1] - gold[k][-1]) <= 1e-10 * abs(gold[k][-1]), k


def test_socal_reference_loop_with_gpu_operator_bitwise(pkg, orc, socal):
    """The reference's loop (the oracle) calling the GPU operator through the
    aprod signature, host vectors in and out on every call: with the
    operator in the reference's order the solve keeps the reference's bits."""
    prob, meta, gold = socal
    it = meta["iterations"]
    o = orc.OracleProblem(prob)
    with pkg.Context(prob, order="reference") as ctx:
        def op(mode, m, n, is_final, iteration):
            ctx.aprod_host(mode, o.y_k, o.y_d, o.x, iteration=iteration, is_final=is_final)
            return 0
        out = o.lsqr(it, op=op)
    assert hashlib.sha256(out["x"].tobytes()).hexdigest() == meta["x_sha256"]
    assert np.array_equal(out["hist"]["alpha"], gold["alpha"])
    assert np.array_equal(out["hist"]["beta"], gold["beta"])
