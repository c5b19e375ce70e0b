"""Independent problems in one persistent launch (pkg.multi.Multi).

Each problem is the reference's FP64 lsqr(); the yardsticks are the oracle
(the reference's algorithm on the CPU) and the one-problem GPU path, both at
the 1e-10 relative bar of the FP64 solver."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def small_uneven(pkg, picks=(0, 4, 9, 14, 19, 23), max_rays=1500):
    cfgs = pkg.multi.uneven_configs()
    out = []
    for i in picks:
        c = dict(cfgs[i], n_rays=min(cfgs[i]["n_rays"], max_rays), iterations=60)
        out.append(pkg.generate(c))
    return out


@pytest.fixture(scope="module")
def uneven(pkg):
    return small_uneven(pkg)


def test_matches_one_problem_path(pkg, uneven):
    with pkg.multi.Multi(uneven) as mp:
        out = mp.solve()
        g, gb = mp.plan()
        assert mp.info()["blocks"] >= len(uneven)
    assert gb[g].min() >= 1 and len(set(g.tolist())) == len(uneven)
    for p, x, h, r in zip(uneven, out["x"], out["hist"], out["results"]):
        with pkg.Context(p) as c:
            ref = c.lsqr(lsqr_iteration=p.iterations)
        assert rel(x, ref["x"]) <= 1e-10
        for f in ("alpha", "beta", "rnorm", "arnorm", "xnorm", "anorm"):
            assert np.allclose(h[f], ref["hist"][f], rtol=1e-10, atol=0), f
        assert r["itn"] == p.iterations
        assert r["rnorm"] == pytest.approx(ref["result"]["rnorm"], rel=1e-10)


@pytest.mark.parametrize("exact", [False, True])
def test_matches_oracle(pkg, orc, uneven, exact):
    """Against the reference's algorithm on the CPU.  (The 10x8x6 problem is
    left out: at 40 iterations a 1e-16 relative change of its b alone moves
    x by 5e-11 to 5e-10, so any regrouping of a norm's sum can cross 1e-10;
    these problems move by less than 1e-13.)"""
    probs = uneven[:3]
    with pkg.multi.Multi(probs) as mp:
        mp.set_exact(exact)
        out = mp.solve()
    for p, x, h in zip(probs, out["x"], out["hist"]):
        o = orc.OracleProblem(p).lsqr(p.iterations)
        assert rel(x, o["x"]) <= 1e-10
        for f in ("alpha", "beta", "rnorm", "arnorm"):
            assert np.allclose(h[f][1:], o["hist"][f][1:], rtol=1e-10, atol=0), f


def test_queues_when_problems_outnumber_blocks(pkg):
    base = pkg.CONFIGS["tiny"]
    with pkg.multi.Multi([pkg.generate("tiny")], iterations=1) as probe:
        count = probe.info()["blocks"] + 64  # the launch's block count plus a queue
    probs = [pkg.generate(dict(base, seed=1000 + i, n_rays=20 + (i % 7) * 10))
             for i in range(count)]
    with pkg.multi.Multi(probs, iterations=12) as mp:
        info = mp.info()
        assert info["count"] > info["blocks"]
        g, gb = mp.plan()
        assert len(set(g.tolist())) == info["blocks"]
        out = mp.solve()
    for i in (0, 261, 519):
        with pkg.Context(probs[i]) as c:
            ref = c.lsqr(lsqr_iteration=12)
        assert rel(out["x"][i], ref["x"]) <= 1e-10


def test_zero_right_hand_side_and_repeat(pkg, uneven):
    p0 = uneven[0]
    zero = pkg.synth.Problem(p0.k_csc, p0.d_csr, p0.d_csc, np.zeros(p0.m_k), p0.x_true, 30)
    with pkg.multi.Multi([zero, uneven[1]], iterations=30) as mp:
        a = mp.solve()
        b = mp.solve()
    assert np.all(a["x"][0] == 0.0) and a["results"][0]["itn"] == 0
    assert np.all(np.isfinite(a["hist"][1]["rnorm"]))
    for xa, xb in zip(a["x"], b["x"]):
        assert np.array_equal(xa, xb)


def test_bounded_wait_returns_timeout(pkg, uneven):
    with pkg.multi.Multi(uneven[:2], iterations=5) as mp:
        assert mp.check_wait(2_000_000) == -8  # PLSQR_ERR_TIMEOUT
        out = mp.solve()  # the context is still usable
        assert all(r["itn"] == 5 for r in out["results"])
        with pytest.raises(pkg._native.PlsqrError):
            mp.set_wait(10)


def test_damped_problems_match_one_problem_path(pkg, uneven):
    """lsqr()'s damp (source/lsqr.c:515-523 rotation) in the persistent launch."""
    probs = uneven[:2]
    with pkg.multi.Multi(probs, damp=0.05) as mp:
        out = mp.solve()
    for p, x, h in zip(probs, out["x"], out["hist"]):
        with pkg.Context(p) as c:
            ref = c.lsqr(lsqr_iteration=p.iterations, damp=0.05)
        assert rel(x, ref["x"]) <= 1e-10
        assert np.allclose(h["rnorm"], ref["hist"]["rnorm"], rtol=1e-10, atol=0)


def test_mixed_sweeps_reach_fp64_solutions(pkg, uneven):
    """FP32 inner / FP64 outer (plsqr_multi_set_mixed): every problem within
    1e-6 of its converged FP64 solution after three sweeps; exact products
    are refused with it, and the FP64 launch afterwards gives the same bits."""
    with pkg.multi.Multi(uneven) as mp:
        base = mp.solve()
        mp.set_mixed(3)
        mixed = mp.solve()
        with pytest.raises(pkg._native.PlsqrError):
            mp.set_exact(True)
        mp.set_mixed(0)
        again = mp.solve()
    for p, xm, x0, x1, r in zip(uneven, mixed["x"], base["x"], again["x"], mixed["results"]):
        assert np.array_equal(x0, x1)
        assert r["itn"] == p.iterations  # the last sweep's LSQR
        with pkg.Context(p) as c:
            xs = c.lsqr(lsqr_iteration=600)["x"]
        assert rel(xm, xs) <= 1e-6, rel(xm, xs)
