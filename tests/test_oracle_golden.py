"""The oracle pinned against the reference program's own outputs.

The golden fixtures under tests/golden were produced by the reference PLSQR3
(compiled from its sources, FP64, one rank) on the generated inputs.  The
oracle must reproduce x, every alpha_k / beta_k and result.txt bit for bit,
and the generator must reproduce the committed inputs byte for byte."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

from conftest import GOLDEN, golden


def _files(case):
    g = golden(case)
    f = dict(g["meta"]["files"])
    f["dir"] = str(GOLDEN / case / "inputs")
    return g, f


def test_generator_reproduces_committed_tiny_inputs(pkg, tmp_path):
    g, _ = _files("tiny")
    prob = pkg.generate("tiny")
    files = pkg.write_files(prob, tmp_path)
    for name, digest in g["meta"]["sha256"].items():
        got = hashlib.sha256((tmp_path / name).read_bytes()).hexdigest()
        assert got == digest, f"{name} differs from the committed input"
        assert (GOLDEN / "tiny" / "inputs" / name).read_bytes() == (tmp_path / name).read_bytes()
    assert files["row_k"] == g["meta"]["files"]["row_k"]


def test_generator_reproduces_grid32_input_digests(pkg, tmp_path):
    g = golden("grid32")
    pkg.write_files(pkg.generate("grid32"), tmp_path)
    for name, digest in g["meta"]["sha256"].items():
        assert hashlib.sha256((tmp_path / name).read_bytes()).hexdigest() == digest, name


@pytest.mark.parametrize("case", ["tiny", "grid32"])
def test_oracle_bitwise_equals_reference(case, pkg, orc, tmp_path):
    g = golden(case)
    if case == "tiny":
        prob = pkg.read_files(_files(case)[1])  # through the product's file readers
    else:
        prob = pkg.generate(case)
    it = g["meta"]["iterations"]
    out = orc.OracleProblem(prob).lsqr(it, result_txt=str(tmp_path / "result.txt"))
    assert np.array_equal(out["x"], g["x"]), "x differs from the reference"
    assert np.array_equal(out["hist"]["alpha"], g["alpha"])
    assert np.array_equal(out["hist"]["beta"], g["beta"])
    assert (tmp_path / "result.txt").read_text() == g["result_txt"]


def test_oracle_thread_count_does_not_change_bits(pkg, orc):
    prob = pkg.generate("tiny")
    g = golden("tiny")
    n0 = orc.get_threads()
    try:
        for t in (1, 3):
            orc.set_threads(t)
            out = orc.OracleProblem(prob).lsqr(g["meta"]["iterations"])
            assert np.array_equal(out["x"], g["x"])
    finally:
        orc.set_threads(n0)


def test_oracle_loop_with_operator_callback_is_bitwise_equal(pkg, orc):
    """The operator-callback form of the oracle's lsqr() (the reference loop
    driving another aprod) with the oracle's own operator behind the
    callback gives the reference's bits, and calls it as lsqr.c does."""
    g = golden("tiny")
    prob = pkg.read_files(_files("tiny")[1])
    it = g["meta"]["iterations"]
    o = orc.OracleProblem(prob)
    calls = []

    def op(mode, m, n, is_final, iteration):
        assert (m, n) == (prob.m_k + prob.m_d, prob.n)
        calls.append((mode, iteration, is_final))
        o.aprod(mode)
        return 0

    out = o.lsqr(it, op=op)
    assert np.array_equal(out["x"], g["x"])
    assert np.array_equal(out["hist"]["alpha"], g["alpha"])
    assert np.array_equal(out["hist"]["beta"], g["beta"])
    assert calls[0] == (2, 0, 0) and len(calls) == 1 + 2 * it
    assert calls[1:3] == [(1, 1, 0), (2, 1, 0)] and calls[-2:] == [(1, it, 1), (2, it, 1)]


def test_oracle_loop_stops_on_operator_error(pkg, orc):
    prob = pkg.generate("tiny")
    o = orc.OracleProblem(prob)

    def op(mode, m, n, is_final, iteration):
        if iteration == 3:
            raise ValueError("operator failed")
        o.aprod(mode)
        return 0

    with pytest.raises(ValueError, match="operator failed"):
        o.lsqr(10, op=op)
    with pytest.raises(RuntimeError, match="oracle_lsqr failed"):
        o.lsqr(10, op=lambda *a: 7)
