"""FP64 parity with the reference on the 96x96x32 grid at full scale.

The golden runs under tests/golden/grid96 (200,000 rays, 1.33e9 kernel
nonzeros: the benchmarked problem) and tests/golden/grid96s (20,000 rays)
were made by the reference program itself (FP64 build, one rank, 300
iterations); the oracle reproduced its x, alpha_k and beta_k bit for bit on
the same inputs and its per-iteration rnorm, arnorm, anorm, xnorm, test1
and test2 are stored beside them (hist.txt).  The inputs are regenerated
here and checked against the digest of the arrays the reference read.

* order="reference" (the reference's order of operations): x (its sha256,
  kept in meta.json) and every iteration's scalars equal the reference's bit
  for bit, all 300 iterations; result.txt is the same text.
* the default order (parallel sums): x within 1e-10 of the reference's (of
  the reference-order x, whose digest is the reference's), or within ten
  times the change of the reference's own x under the one-ulp probe below
  where that is larger: on the 200,000-ray problem 300 iterations stop short
  of convergence (1e-6 of the solution takes ~376), and the reference's x
  there moves by 1.2e-6 when every element of b_k is raised by one ulp.
  Per iteration the bar is 1e-10 over the iterations where the reference's
  own scalars are well conditioned: ulp.txt records how far they move when
  every element of b_k is raised by one ulp (a change of the size of the
  rounding differences between two summation orders).  That change stays at
  the level of roundoff for the first iterations, then grows about a
  hundredfold per iteration until alpha_k and beta_k have lost every digit
  (on the 20,000-ray problem past 1e-12 at iteration 13 and at 1e-2 by 18).
  No evaluation in another order can follow the reference's scalars there;
  the iterations before that change first exceeds 1e-12 are held to 1e-10,
  and the converged quantities (x, the final rnorm and xnorm) at the end."""
from __future__ import annotations

import hashlib
import importlib.util
import re

import numpy as np
import pytest

from conftest import GOLDEN, golden, rel

pytestmark = pytest.mark.gpu

LSQR_TOL = 1e-10
HIST_KEYS = ("rnorm", "arnorm", "anorm", "xnorm", "test1", "test2")
CASES = ["grid96s", "grid96"]


def _array_digest(prob) -> str:
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.array_digest(prob)


def rel_each(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-300)


def golden_hist(case):
    h = np.loadtxt(GOLDEN / case / "hist.txt")
    return {k: h[:, 1 + i] for i, k in enumerate(HIST_KEYS)}


def stable_prefix(case, limit=1e-12) -> int:
    """Iterations 0..k-1 where a one-ulp raise of every element of b moves
    none of the reference's alpha, beta, rnorm, arnorm by more than `limit`."""
    u = np.loadtxt(GOLDEN / case / "ulp.txt")
    bad = np.nonzero(np.max(u[:, 1:], axis=1) > limit)[0]
    return int(bad[0]) if bad.size else u.shape[0]


@pytest.fixture(scope="module")
def big(pkg):
    cache = {}

    def get(case):
        if case not in cache:
            cache.clear()  # one full-size problem in host memory at a time
            prob = pkg.generate(case)
            g = golden(case)
            assert prob.meta["nnz_k"] == g["meta"]["nnz_k"]
            assert _array_digest(prob) == g["meta"]["array_sha256"], \
                "inputs differ from the golden run's"
            cache[case] = prob
        return cache[case]

    return get


@pytest.fixture(scope="module")
def ref_order(pkg, big):
    """The reference-order solve of a case (once per module)."""
    cache = {}

    def get(case, tmp_path):
        if case not in cache:
            g = golden(case)
            txt = tmp_path / "result.txt"
            with pkg.Context(big(case), order="reference") as ctx:
                out = ctx.lsqr(lsqr_iteration=g["meta"]["iterations"], result_txt=str(txt))
            out["result_txt"] = txt.read_text()
            cache.clear()
            cache[case] = out
        return cache[case]

    return get


def check_result_txt(path, g):
    """Same lines as the reference's result.txt, numbers aside."""
    mine, theirs = path.read_text().splitlines(), g["result_txt"].splitlines()
    assert len(mine) == len(theirs)
    num = re.compile(r"[-+]?\d+\.\d+e[-+]\d+")
    for a, b in zip(mine, theirs):
        assert num.sub("#", a) == num.sub("#", b)


@pytest.mark.parametrize("case", CASES)
def test_reference_order_bitwise_fullsize(case, ref_order, tmp_path):
    g = golden(case)
    gh = golden_hist(case)
    it = g["meta"]["iterations"]
    out = ref_order(case, tmp_path)
    h = out["hist"]
    assert hashlib.sha256(out["x"].tobytes()).hexdigest() == g["meta"]["x_sha256"]
    assert np.array_equal(h["alpha"], g["alpha"])
    assert np.array_equal(h["beta"], g["beta"])
    for k in HIST_KEYS:
        assert np.array_equal(h[k][1:], gh[k][1:]), k
    assert out["result_txt"] == g["result_txt"]
    print(f"{case}: reference order, {it} iterations: bitwise equal to the reference, "
          f"{out['result']['seconds']:.2f} s")


@pytest.mark.parametrize("case", CASES)
def test_fast_order_matches_reference_fullsize(case, pkg, big, ref_order, tmp_path):
    g = golden(case)
    gh = golden_hist(case)
    prob = big(case)
    xr = ref_order(case, tmp_path)["x"]
    assert hashlib.sha256(xr.tobytes()).hexdigest() == g["meta"]["x_sha256"]
    it = g["meta"]["iterations"]
    ks = stable_prefix(case)
    with pkg.Context(prob) as ctx:
        out = ctx.lsqr(lsqr_iteration=it, result_txt=str(tmp_path / "result.txt"))
    h = out["hist"]
    dev = {"alpha": rel_each(h["alpha"], g["alpha"]), "beta": rel_each(h["beta"], g["beta"])}
    for k in HIST_KEYS:
        dev[k] = np.concatenate([[0.0], rel_each(h[k][1:], gh[k][1:])])
    ex = rel(out["x"], xr)
    # the reference's own sensitivity, where the golden run recorded it
    x_bar = max(LSQR_TOL, 10.0 * g["meta"].get("ulp_x_rel", 0.0))
    u_last = np.loadtxt(GOLDEN / case / "ulp.txt")[-1]
    r_bar = max(LSQR_TOL, 10.0 * u_last[3])
    print(f"{case}: default order, x within {ex:.2e} of the reference; per iteration, "
          f"k < {ks}: " + ", ".join(f"{k} {np.max(v[:ks]):.1e}" for k, v in dev.items())
          + "; all k: " + ", ".join(f"{k} {np.max(v):.1e}" for k, v in dev.items())
          + f"; bars: x {x_bar:.1e}, final rnorm {r_bar:.1e}")
    assert ex <= x_bar
    assert ks >= 10, "the reference is ill-conditioned from the first iterations"
    for k, v in dev.items():
        assert np.max(v[:ks]) <= LSQR_TOL, (k, int(np.argmax(v[:ks])), float(np.max(v[:ks])))
    # converged quantities at the end of the solve
    assert dev["rnorm"][-1] <= r_bar
    assert dev["xnorm"][-1] <= x_bar
    check_result_txt(tmp_path / "result.txt", g)
