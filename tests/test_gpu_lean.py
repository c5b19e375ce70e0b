"""A lean FP64 context (plsqr_opts.lean): once the unit layouts hold both
products, the by-row and by-column copies of K are released.  The solve and
the operator give the same bits as a full context with less device memory;
the batched solver, which reads those copies, refuses; lean needs an FP64
context in the fast order."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PLSQR_ERR_STATE = -7


def test_lean_context_same_bits_less_memory(pkg, problems):
    prob = problems("grid32")
    rng = np.random.default_rng(5)
    yk, yd, x = rng.standard_normal(prob.m_k), rng.standard_normal(prob.m_d), rng.standard_normal(prob.n)
    outs, mem, ops = {}, {}, {}
    for lean in (False, True):
        with pkg.Context(prob, lean=lean) as ctx:
            outs[lean] = ctx.lsqr(lsqr_iteration=60)
            mem[lean] = ctx.info()["device_bytes"]
            a, b, c = yk.copy(), yd.copy(), x.copy()
            ctx.aprod_host(1, a, b, c)
            ctx.aprod_host(2, a, b, c)
            ops[lean] = (a, b, c)
            if lean:
                with pytest.raises(pkg._native.PlsqrError) as e:
                    ctx.batch_lsqr(np.stack([prob.b_k, prob.b_k]), sweeps=1, inner=5)
                assert e.value.code == PLSQR_ERR_STATE
                # the context still solves after the refusal
                again = ctx.lsqr(lsqr_iteration=60)
                assert np.array_equal(again["x"], outs[True]["x"])
    assert np.array_equal(outs[True]["x"], outs[False]["x"])
    for k in ("alpha", "beta", "rnorm", "arnorm"):
        assert np.array_equal(outs[True]["hist"][k], outs[False]["hist"][k]), k
    for u, v in zip(ops[True], ops[False]):
        assert np.array_equal(u, v)
    # both copies of K go: 4-byte index + 8-byte value per nonzero each
    nnz = prob.meta["nnz_k"]
    assert mem[False] - mem[True] >= 24 * nnz


def test_lean_needs_fast_fp64(pkg, problems):
    prob = problems("tiny")
    for kw in (dict(order="reference"), dict(precision="mixed")):
        with pytest.raises(pkg._native.PlsqrError):
            pkg.Context(prob, lean=True, **kw)
